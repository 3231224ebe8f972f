/*
 * houghline_gb300.h -- C ABI of the GB300 HoughLine path.
 *
 * Plain C types only (pointers, sizes, POD structs); a CUDA stream is passed
 * as `void *` holding a cudaStream_t (NULL = the legacy default stream).
 * Every call returns an OpenCUDA ErrorCode (okano_3_0/ErrorCode.h:16-56):
 *   HL_NO_ERROR 0, HL_INVALID_DATA -1, HL_NULL_POINTER -2, HL_OP_OVERFLOW -3,
 *   HL_OUT_OF_MEM -6, HL_CUDA_ERROR -7, HL_UNIMPLEMENT -998.
 * CUDA failures never leak a raw cudaError_t (the reference sometimes does,
 * okano_3_0/HoughLine.cu:399,464).
 *
 * A handle owns its device workspace (grown on demand, reused across calls)
 * and the cos/sin table for its detheta.  One handle serves one host thread
 * and one stream at a time, like the reference's HoughLine object.
 */
#ifndef HOUGHLINE_GB300_H
#define HOUGHLINE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HL_NO_ERROR       0
#define HL_INVALID_DATA  -1
#define HL_NULL_POINTER  -2
#define HL_OP_OVERFLOW   -3
#define HL_OUT_OF_MEM    -6
#define HL_CUDA_ERROR    -7
#define HL_UNIMPLEMENT   -998

/* Largest ROI side: coordinates are packed as two 16-bit halves. */
#define HL_MAX_SIDE 65535

typedef struct hl_handle hl_handle;

/* HoughLine members, okano_3_0/HoughLine.h:86-115 (defaults :120-124:
 * detheta = M_PI/180, derho = 1, threshold = 90, thresang = 5 deg,
 * thresdis = 50). */
typedef struct hl_params {
    double detheta;   /* angle step, radians; numtheta = (int)(M_PI/detheta) */
    double derho;     /* distance step */
    int threshold;    /* a peak needs votes > threshold */
    float thresang;   /* merge: angle difference below this is one line */
    int thresdis;     /* merge: distance difference below this is one line */
} hl_params;

/* LineParam, okano_3_0/HoughLine.h:70-74 (same 12-byte layout). */
typedef struct hl_line {
    float angle;      /* radians, k * detheta */
    int distance;     /* rho bin, with the reference's +1 on negative bins */
    int votes;        /* exact int32 count of the bin */
} hl_line;

/* An 8-bit image and its ROI, the fields of Image + ImageCuda
 * (okano_3_0/Image.h:44-78): data points at pixel (0,0) of the full image,
 * the ROI is [roi_x1, roi_x2) x [roi_y1, roi_y2) (okano_3_0/Image.h:218-258). */
typedef struct hl_image_desc {
    const uint8_t *data;
    size_t pitch;     /* bytes per row */
    int width, height;
    int roi_x1, roi_y1, roi_x2, roi_y2;
} hl_image_desc;

/* Shape of the vote work for one image (filled by hl_geometry). */
typedef struct hl_geom {
    int numtheta;     /* T */
    int theta_pad;    /* T rounded up to 32 (accumulator row length) */
    int rho_min;      /* first rho bin of the accumulator */
    int numrho;       /* R = 2 * floor(diag / derho + 0.5) + 1 */
    int ref_numrho;   /* the reference's numrho, okano_3_0/HoughLine.cu:670 */
    int tiles_x, tiles_y;
} hl_geom;

/* Replaces the HoughLine constructors, okano_3_0/HoughLine.h:116-156
 * (params == NULL -> defaults). */
int hl_create(hl_handle **out, const hl_params *params);
int hl_destroy(hl_handle *h);
/* setDeTheta/setDeRho/setThreshold/setThresAng/setThresDis,
 * okano_3_0/HoughLine.h:158-262. */
int hl_set_params(hl_handle *h, const hl_params *params);
int hl_get_params(const hl_handle *h, hl_params *params);

/* Geometry of a w x h ROI under the handle's parameters. */
int hl_geometry(const hl_handle *h, int w, int h_, hl_geom *g);

/* cos/sin table, theta_k = (float)(k * detheta), evaluated on the GPU with
 * CUDA's cosf/sinf -- exactly what the reference vote kernel evaluates per
 * (pixel, k) (okano_3_0/HoughLine.cu:115-119).  Copies T floats each. */
int hl_trig_table(hl_handle *h, float *cos_host, float *sin_host);

/* HoughLine::houghLine(inimg, NULL, linesmax, lineparam),
 * okano_3_0/HoughLine.cu:635-955.  img->data is a DEVICE pointer; lines is a
 * HOST array of *linesmax records.  On return *linesmax = min(lines found,
 * *linesmax).  Synchronises `stream`. */
int hl_plain(hl_handle *h, const hl_image_desc *img, int *linesmax,
             hl_line *lines, void *stream);

/* Same, asynchronous and device-resident: writes min(found, linesmax)
 * records to lines_dev and the count to *count_dev, no host sync.  The
 * result is valid once `stream` reaches this point.  Launch errors are
 * returned; in-kernel errors are reported by hl_last_status. */
int hl_plain_async(hl_handle *h, const hl_image_desc *img, int linesmax,
                   hl_line *lines_dev, int *count_dev, void *stream);

/* Device status word of the last asynchronous call (0 = fine); syncs. */
int hl_last_status(hl_handle *h, int *status, void *stream);

/* Batched plain HoughLine: nimg independent DEVICE images (each with its own
 * size and ROI) through one compaction, one persistent vote launch over the
 * (image, theta slice, rho window) work queue, one peak pass and one
 * finalize CTA per image.  Every image gets the result hl_plain would give
 * it (same vote rule, its own rho range, the handle's theta step, thresdis
 * and thresang); thresholds[i] replaces the handle's vote threshold for
 * image i when thresholds is not NULL.  The reference has no batched entry
 * point: a caller loops over HoughLine::houghLine (okano_3_0/HoughLine.cu:
 * 635-955), as the tiled HoughRec callers do (okano_3_0/HoughRec.cu:716-760).
 *
 * hl_batch: lines is a HOST array of nimg * linesmax records (image i at
 * i * linesmax), counts a HOST array of nimg line counts.  Synchronises.
 * hl_batch_async: the same into DEVICE arrays, no host sync (the per-image
 * tables are staged in pinned memory owned by the handle, reused once the
 * previous batch call on the handle has read them); in-kernel errors are
 * reported by hl_last_status.
 * With hl_set_batch_graph(h, 1) a call whose image sizes, linesmax, output
 * pointers and launch shape equal the previous call's replays a captured
 * CUDA graph of the whole pipeline instead of launching its kernels one by
 * one (the first such call captures it). */
int hl_batch(hl_handle *h, const hl_image_desc *imgs, int nimg,
             const int *thresholds, int linesmax, hl_line *lines, int *counts,
             void *stream);
int hl_batch_async(hl_handle *h, const hl_image_desc *imgs, int nimg,
                   const int *thresholds, int linesmax, hl_line *lines_dev,
                   int *counts_dev, void *stream);
int hl_set_batch_graph(hl_handle *h, int enable);

/* The tiled caller of okano_3_0/HoughRec.cu:716-760 as one hl_batch call:
 * img (its data, pitch and size; its own ROI is ignored, as the reference
 * overwrites it) in piecenum x piecenum cells of cell_x = width / piecenum by
 * cell_y = height / piecenum pixels, cell (x, y) with ROI [x cell_x,
 * x cell_x + cell_x - 1) x [y cell_y, y cell_y + cell_y - 1) (the
 * reference's exclusive end drops the cell's last column and row).  lines /
 * counts: HOST arrays of piecenum^2 * linesmax records and piecenum^2 counts,
 * cell y * piecenum + x first; line parameters are in the cell's local
 * coordinates, as the reference's per-cell houghLine calls return them. */
int hl_tiles(hl_handle *h, const hl_image_desc *img, int piecenum, int linesmax,
             hl_line *lines, int *counts, void *stream);

/* Autotuner (no reference counterpart): times hl_batch_async on the given
 * images for every candidate vote-kernel shape (rho-window rows x threads
 * per CTA), keeps the fastest with hl_set_vote_shape and reports it.
 * tried[] (optional, up to max_tried entries) receives every candidate and
 * its mean milliseconds per batch; *ntried their number. */
typedef struct hl_tune_entry {
    int window_rows;
    int threads;
    float ms;
} hl_tune_entry;
int hl_autotune(hl_handle *h, const hl_image_desc *imgs, int nimg,
                const int *thresholds, int linesmax, hl_tune_entry *best,
                hl_tune_entry *tried, int max_tried, int *ntried,
                void *stream);

/* HoughLine::houghLineCor / houghLine(NULL, guidingset, ...),
 * okano_3_0/HoughLine.cu:352-632: votes over an interleaved (x, y) int list
 * in DEVICE memory.  The accumulator covers the set's bounding box from the
 * origin, so every coordinate votes in range (the reference sizes it by the
 * box extent only, :374-375, and can index outside its buffer). */
int hl_plain_points(hl_handle *h, const int *xy_dev, int n, int *linesmax,
                    hl_line *lines, void *stream);

/* Stage (a): compact the ROI's 255-pixels into packed (x | y << 16) ROI
 * coordinates, tile-major (tiles of 128 x 32 pixels in raster order, raster
 * order inside a tile).  pts_dev holds w*h entries, tile_off_dev
 * tiles_x*tiles_y + 1; *count_dev gets the number of points. */
int hl_compact(hl_handle *h, const hl_image_desc *img, uint32_t *pts_dev,
               int *tile_off_dev, int *count_dev, void *stream);

/* Stage (a) without allocating: the same compaction as hl_compact, for
 * callers that may not call cudaMalloc after start-up (their device memory is
 * owned by another memory manager or fixed by a budget, or an allocation
 * would stall a latency-bound loop).  No counterpart in the reference.  The
 * look-back scratch lives in a static device array of this library (one
 * state per group of four tiles: about 128 KiB on every device that loads
 * it, kept until exit), so the ROI may cover at most 65536 tiles of 128 x 32
 * pixels (HL_OP_OVERFLOW beyond).  The first call on a device looks up that
 * array's device address and should come before any stream capture.  No
 * handle is needed; every call shares the one array and clears what it
 * uses, so calls that overlap on the GPU (two streams at once) race.
 * Asynchronous on `stream`; a device-side wait that gave up is reported by
 * hl_compact_noalloc_status, which callers should check before using the
 * points. */
int hl_compact_noalloc(const hl_image_desc *img, uint32_t *pts_dev,
                       int *tile_off_dev, int *count_dev, void *stream);

/* Status word of the last hl_compact_noalloc call on this device (0 = fine,
 * bit 0x1 set = a look-back wait gave up and the tile offsets are not
 * valid).  Synchronises `stream`; allocates nothing. */
int hl_compact_noalloc_status(int *status, void *stream);

/* Stages (a)+(b): the int32 accumulator of the ROI in the tight layout
 * acc[(rho - rho_min) * T + k] (R * T ints, DEVICE), for parity checks. */
int hl_accumulator(hl_handle *h, const hl_image_desc *img, int32_t *acc_dev,
                   void *stream);

/* Same accumulator in the reference layout (okano_3_0/HoughLine.cu:683-705):
 * (T + 2) x (ref_numrho + 2) ints with a zero border, DEVICE. */
int hl_accumulator_ref_layout(hl_handle *h, const hl_image_desc *img,
                              int32_t *ref_dev, void *stream);

/* Stage (c) alone on a tight-layout accumulator in DEVICE memory:
 * peaks + rank + decode + merge for a w x h ROI.  Host result like hl_plain. */
int hl_lines_from_accumulator(hl_handle *h, const int32_t *acc_dev, int w,
                              int h_, int *linesmax, hl_line *lines,
                              void *stream);

/* Vote-kernel launch shape: rows of the rho window held per CTA (0 = auto)
 * and threads per CTA (0 = auto). */
int hl_set_vote_shape(hl_handle *h, int window_rows, int threads);

/* Shared-memory int32 atomicAdd ceiling of this GPU: conflict-free atomics
 * per second over all SMs, measured by a micro-kernel (iters per thread). */
int hl_measure_smem_atomic_peak(int iters, double *atomics_per_s,
                                void *stream);

/* Per-stage device timing with CUDA events on the call's stream: after
 * hl_profile(h, 1), every hl_plain / hl_plain_async records events around
 * compact, vote, peaks and finalize; hl_profile_read adds up the elapsed
 * milliseconds per stage (stage_ms[4]) over the recorded calls, returns their
 * number and starts a new record. */
int hl_profile(hl_handle *h, int enable);
int hl_profile_read(hl_handle *h, double *stage_ms, int *calls);

/* Number of kernels the last hl_plain / hl_plain_async call launched. */
int hl_last_launch_count(const hl_handle *h);

/* HoughLine::houghLineImg (okano_3_0/HoughLine.cu:958-1345) on DEVICE
 * images: both ROIs are cut to the smaller width and height (:1101-1109),
 * the lines are found as in hl_plain (records to the HOST array `lines`),
 * then drawn into the output ROI: a pixel becomes 255 where
 * (int)(fl(c*cos a) + fl(r*sin a)) equals a line's distance (:216-249);
 * other output pixels are left as they are.  Synchronises `stream`. */
int hl_plain_draw(hl_handle *h, const hl_image_desc *in,
                  const hl_image_desc *out, int *linesmax, hl_line *lines,
                  void *stream);

/* The drawing step of houghLineImg alone: nlines HOST records drawn into the
 * ROI of a DEVICE image (_houghoutKer, okano_3_0/HoughLine.cu:216-249).
 * Synchronises `stream`. */
int hl_draw_lines(hl_handle *h, const hl_image_desc *out,
                  const hl_line *lines, int nlines, void *stream);

/* HoughLine::realLine (okano_3_0/HoughLine.cu:1377-1462): counts the ROI's
 * 255-pixels inside the segment's bounding box grown by (int)threshold whose
 * distance to the line through (x1,y1)-(x2,y2) is below (int)threshold;
 * *is_real = count > (int)|segment| * thresperc.  Coordinates are ROI-local.
 * pointnum (optional) receives the count.  Synchronises `stream`. */
int hl_real_line(hl_handle *h, const hl_image_desc *img, int x1, int y1,
                 int x2, int y2, float threshold, float thresperc,
                 int *is_real, int *pointnum, void *stream);

/* Synthetic scenes (seeded, integer-only; identical on every host). */
typedef struct hl_scene_params {
    int width, height;
    int nseg;
    int len_min, len_max;
    int salt_ppm;
    int nbezier;
    uint64_t seed;
} hl_scene_params;
int hl_synth_scene(const hl_scene_params *p, uint8_t *img, long pitch);
int hl_synth_spec(int kind, uint64_t seed, int n, hl_scene_params *out);

#ifdef __cplusplus
}
#endif
#endif
