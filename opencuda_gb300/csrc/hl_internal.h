/*
 * hl_internal.h -- kernel argument blocks and launchers shared by the
 * translation units of libhoughline_gb300.so (not part of the C ABI).
 */
#ifndef HL_INTERNAL_H
#define HL_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "houghline_gb300.h"
#include "hl_circle.h"

#include <utility>

/* Compaction tiles: 128 x 32 pixels; one CTA of 256 threads reads one tile,
 * 16 pixels (one 16-byte vector) per thread. */
#define HL_TILE_W 128
#define HL_TILE_H 32
#define HL_COMPACT_THREADS 256
/* Tiles per compaction CTA (one look-back per group). */
#define HL_COMPACT_GROUP 4
/* Theta slice = one warp: lane i owns theta k0 + i. */
#define HL_SLICE 32

/* Bits of the device status word. */
#define HL_ST_LOOKBACK_TIMEOUT 0x1
#define HL_ST_CAND_OVERFLOW 0x2
#define HL_ST_RHO_OUT_OF_RANGE 0x4
#define HL_ST_MERGE_OVERFLOW 0x8
#define HL_ST_VOTE_TIMEOUT 0x10
#define HL_ST_CNN_TIMEOUT 0x20

/* Result block written by the finalize kernel (device) and copied to the
 * host in one transfer. */
typedef struct hl_result_hdr {
    int count;    /* lines written = min(survivors, linesmax) */
    int status;   /* HL_ST_* bits seen during this call */
    int ncand;    /* peaks found */
    int pad;
} hl_result_hdr;

typedef struct hl_roi {
    const uint8_t *base;  /* ROI origin */
    long pitch;
    int w, h;
} hl_roi;

/* One image of a batched compaction: its tiles occupy [tile_base, +ntiles)
 * of the batch's tile_off array, its 4-tile groups [group_base, +ngroups) of
 * the batch's group space, and its points start at pts_base of the batch's
 * point array (room for every pixel plus one pad per tile).  Prefixes and
 * tile offsets are per image: an image's groups wait only for each other. */
typedef struct hl_compact_img {
    hl_roi roi;
    int tiles_x, ntiles;
    int tile_base, group_base, ngroups;
    int pad;
    long long pts_base;
} hl_compact_img;

typedef struct hl_compact_args {
    /* one image (imgs == NULL) ... */
    hl_roi roi;
    int tiles_x, ntiles;
    /* ... or a batch: group g belongs to image group_img[g] */
    const hl_compact_img *imgs;
    const int *group_img;
    int nimg, ngroups;
    unsigned long long *tile_state;  /* [ntiles], epoch-tagged */
    unsigned int *ticket;            /* monotonically increasing counter */
    unsigned int ticket_base;        /* value of *ticket at launch */
    unsigned int epoch;              /* 1..2^30-1, distinct per launch */
    uint32_t *pts;                   /* out: packed x | y << 16, or NULL */
    float2 *pts_f2;                  /* out: (x, y) as floats, or NULL */
    int *tile_off;                   /* out: [ntiles + 1] */
    int *count;                      /* out: total points */
    int *status;
} hl_compact_args;


/* One image of a vote launch. */
typedef struct hl_vote_img {
    const float2 *pts;        /* (x, y) of every edge point, tile-major */
    const int *tile_off;      /* the image's [ntiles + 1] tile offsets */
    /* admitted tiles of every (slice, window) block: bit t % 32 of word
     * [block][t / 32] (hl_launch_tile_masks; they depend on the geometry
     * only) */
    unsigned *tmask;
    int ntiles, tiles_x;
    int w, h;                 /* ROI size (tile clipping) */
    int rho_min, R;
    int nwin;                 /* rho windows of win_rows rows */
    int threshold;            /* peak threshold: bins above it are noted */
    int32_t *acc;             /* [R][Tp] */
} hl_vote_img;

/* Peak candidates of a launch: every accumulator bin above its image's
 * threshold, noted as image << 32 | (row * T + theta) when its final count
 * is stored (the vote's block store, the merge of a split block).  A
 * counter past cap means some were not noted: the peak pass then scans
 * every accumulator instead.  The counter is zero at the vote's start (the
 * batch clears it with its other counters); e == NULL: nothing is noted. */
typedef struct hl_cand_list {
    unsigned long long *e;
    int *count;               /* cleared by the compaction launch */
    int cap;
    int pad;
} hl_cand_list;

typedef struct hl_vote_args {
    const hl_vote_img *imgs;  /* per image, or NULL: the one image img0 */
    hl_vote_img img0;
    const float *cosv, *sinv; /* [theta_pad] */
    int T, Tp;
    int win_rows;             /* rho window per work item */
    float irho;
    int *status;
    /* persistent scheduling: work items are taken in the order items[]
     * (heaviest first) from a monotonically increasing counter.  An item is
     * one part of a (slice, window) block of one image: .x = block | image
     * << 16 with block = slice + nslices * window, .y = part | nparts << 16,
     * .z = the part's scratch slot when nparts > 1, .w = 0.  A whole block
     * is stored into the accumulator; a part of a split block stores its
     * counts to its slot, and hl_merge_kernel adds the parts' slots into the
     * block afterwards. */
    const int4 *items;
    int nitems;
    unsigned *work;           /* counter */
    unsigned work_base;       /* its value at launch */
    int4 *scratch;            /* slots of win_rows x HL_SLICE counts */
    /* nonzero: a slot holds 16-bit counts (two per word; the host sets it
     * when no bin can reach 2^16 votes, see hl_part16_ok), half the bytes */
    int part16;
    hl_cand_list cand;
} hl_vote_args;

/* A split vote block: its accumulator region (rows x 8 int4 from off4, rows
 * pitch4 apart, first theta k0) is the sum of nparts scratch slots from
 * slot0 on. */
typedef struct hl_merge_region {
    long long off4;
    int rows, k0;
    int slot0, nparts;
    int w0;                   /* first row of the block in its image */
    int img;                  /* its image */
    int pad[2];
} hl_merge_region;

struct hl_peak_img;

typedef struct hl_merge_args {
    int4 *acc;
    int pitch4;
    int T;
    const int4 *scratch;
    long long slot4;          /* int4 per scratch slot */
    const hl_merge_region *regs;
    int nreg;
    int part16;               /* slots hold 16-bit counts (hl_vote_args) */
    /* the peak threshold of region r: pimgs[r.img].threshold, or thr0 */
    const struct hl_peak_img *pimgs;
    int thr0;
    hl_cand_list cand;
} hl_merge_args;

/* Can a split part's counts be kept in 16 bits?  A bin of one rho bin width
 * derho (the rho-0 bin spans two, truncation toward zero) holds the pixels of
 * a strip of width <= 2 derho across the ROI: fewer than (2 derho + 2)(w + h)
 * of them. */
static inline int hl_part16_ok(double derho, int w, int h)
{
    return (2.0 * derho + 2.0) * ((double)w + (double)h) < 65535.0;
}
/* int4 per scratch slot of a launch */
#ifdef __CUDACC__
__host__ __device__
#endif
static inline long long hl_slot4(int win_rows, int part16)
{
    return (long long)win_rows * (HL_SLICE / 4) / (part16 ? 2 : 1);
}

/* Tiles the allocation-free compaction entry point can serve. */
#define HL_NOALLOC_MAX_TILES 65536

/* Vote-kernel staging: points per consumer warp per batch, points per ring
 * slot (at most 31 consumer warps), ring slots, tiles per coarse-filter
 * group. */
#define HL_VOTE_PPW 64
#define HL_VOTE_CHUNK (HL_VOTE_PPW * 32)
#define HL_VOTE_SLOTS 3
#define HL_VOTE_TG 4096
/* largest rho window (rows) one CTA can hold next to its staging */
int hl_vote_max_rows(void);

/* One image of a peak pass. */
typedef struct hl_peak_img {
    const int32_t *acc;       /* [R][Tp] */
    unsigned long long *keys; /* votes << 32 | ~tight_index */
    int *ncand;
    int R, cap;
    int threshold;            /* votes must exceed it */
    int pad;
} hl_peak_img;

/* rows of an accumulator one peak-pass chunk covers (several images), int4
 * of a unit of one image's accumulator, threads of a peak-pass CTA */
#define HL_PEAK_ROWS 16
#define HL_PEAK_THREADS 256
#define HL_PEAK_LOADS 4           /* 16-byte loads in flight per thread */
#define HL_PEAK_FLAT (HL_PEAK_LOADS * HL_PEAK_THREADS)
#define HL_PEAK_CTAS_PER_SM 6

typedef struct hl_peak_args {
    const hl_peak_img *imgs;  /* per image, or NULL: the one image img0 */
    hl_peak_img img0;
    const int2 *chunks;       /* {image, first row}, HL_PEAK_ROWS rows each;
                                 NULL: unit c is int4 c * HL_PEAK_FLAT.. of
                                 img0's accumulator */
    int nchunks;
    int T, Tp;
    int *status;
    /* the bins above the threshold, noted by the vote and the merge; when
     * they all fit, only they are tested (no scan of the accumulators) */
    hl_cand_list cand;
} hl_peak_args;

/* One image of a finalize launch (one CTA per image). */
typedef struct hl_final_img {
    const unsigned long long *keys;
    int *ncand;               /* read, then reset to 0 for the next call */
    int cap;
    int rho_min, ref_numrho;
    int pad;
    hl_line *lines;           /* out: [linesmax] */
    int *count_out;           /* out: lines written, or NULL */
} hl_final_img;

typedef struct hl_final_args {
    const hl_final_img *imgs; /* per image (CTA), or NULL: the one image img0 */
    hl_final_img img0;
    int T;
    double detheta;
    int thresdis;
    float thresang;
    int linesmax;
    hl_result_hdr *hdr;       /* out (one image), or NULL */
    int *status;              /* read; reset to 0 when hdr is set */
} hl_final_args;

/* The whole plain path of one small image in one cluster launch (see
 * hl_small_kernel): usable when Tp / 32 <= HL_SMALL_MAX_CTAS and the R x 32
 * accumulator slice plus its dump row fit one CTA's shared memory. */
#define HL_SMALL_MAX_CTAS 8
typedef struct hl_small_args {
    hl_roi roi;
    float2 *pts;              /* w * h entries of scratch (global) */
    const float *cosv, *sinv; /* [Tp] */
    int T, Tp, R, rho_min;
    float irho;
    int threshold;
    hl_final_args fin;        /* keys, counters, result records */
    float scale;              /* (float)(1 / (T + 2)), the reference decode */
} hl_small_args;
int hl_small_fits(int T, int Tp, int R);
cudaError_t hl_launch_small(const hl_small_args *a, cudaStream_t s);

/* launchers (return cudaGetLastError() after the launch) */
cudaError_t hl_launch_trig(float *cosv, float *sinv, int T, int Tp,
                           double detheta, cudaStream_t s);
#ifdef __CUDACC__
/* Programmatic dependent launch: the pipeline's kernels are launched with
 * programmatic stream serialization, so a kernel's grid can be set up while
 * its predecessor drains.  Each kernel waits for its predecessor's completion
 * (and memory) before it touches global memory, then lets its own successor
 * launch.  Both are no-ops for a kernel launched the ordinary way. */
__device__ __forceinline__ void hl_pdl_begin()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

/* launch `kernel` with programmatic stream serialization (and, if coop, as a
 * cooperative launch) */
template <typename... Params, typename... Args>
static inline cudaError_t hl_launch_pdl(void (*kernel)(Params...), dim3 grid, dim3 block,
                                        size_t smem, cudaStream_t s, bool coop,
                                        Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    at[1].id = cudaLaunchAttributeCooperative;
    at[1].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = coop ? 2 : 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}
#endif
/* HoughCircle (hl_circle.cu) */
#define HL_CIRCLE_MAXCAND 4096
/* One CTA per (accumulator tile, radius): the tile and a one-cell apron are
 * counted in shared memory from the points of the halo (the compaction tiles
 * within the radius of the tile); then the interior is written to acc and/or
 * its local maxima appended to keys. */
#define HL_CIRCLE_TW 256
#define HL_CIRCLE_TH 192
/* One image of a circle batch: its points and tile offsets (the batch
 * compaction's region of the image), its ROI, its candidate keys and
 * counters, its result records, and the first CTA of its tile launch. */
typedef struct hl_circle_img {
    const float2 *pts;
    const int *tile_off;
    int ctiles_x, ctiles_y;
    int w, h;
    int ntx, nty;
    int roi_x, roi_y;
    int cta_base;
    int pad;
    unsigned long long *keys; /* [HL_CIRCLE_MAXCAND] */
    int *ncand;               /* [ncand, status] */
    hl_circle *out;
    hl_result_hdr *hdr;
} hl_circle_img;
typedef struct hl_circle_tile_args {
    /* a batch: the CTA's image is the last with cta_base <= blockIdx.x, and
     * its fields replace pts .. nty, keys, ncand and status below */
    const hl_circle_img *imgs;
    int nimg;
    int nctas;                /* CTAs of a batch (every image's tiles x radii) */
    const float2 *pts;        /* the compaction's points (odd tiles padded) */
    const int *tile_off;      /* [ctiles_x * ctiles_y + 1] */
    int ctiles_x, ctiles_y;   /* compaction tiles (HL_TILE_W x HL_TILE_H) */
    int w, h;                 /* ROI */
    int rmin, nr;
    int ntx, nty;             /* accumulator tiles */
    int32_t *acc;             /* [nr][h][w], or NULL */
    int threshold;
    unsigned long long *keys; /* votes << 32 | ~index, or NULL */
    int *ncand;
    int cap;
    int *status;
} hl_circle_tile_args;
typedef struct hl_circle_final_args {
    /* a batch: CTA i takes image i's keys, counters, ROI and outputs */
    const hl_circle_img *imgs;
    const unsigned long long *keys;
    int *ncand;
    int w, h, rmin;
    float dist_thres;
    int r_thres;
    int circlemax;
    int roi_x, roi_y;         /* added to the centres */
    hl_circle *out;
    hl_result_hdr *hdr;
    int *status;
} hl_circle_final_args;
cudaError_t hl_launch_circle_tiles(const hl_circle_tile_args *a, cudaStream_t s);
/* grid: one CTA, or nimg CTAs for a batch */
cudaError_t hl_launch_circle_final(const hl_circle_final_args *a, int nimg, cudaStream_t s);

cudaError_t hl_launch_compact(const hl_compact_args *a, cudaStream_t s);
/* one image (a->imgs == NULL) with hl_compact_persist_ctas(ntiles, sms) CTAs
 * in a cooperative launch (0: too many to be resident at once), each adding
 * one to the ticket word */
int hl_compact_persist_ctas(int ntiles, int sms);
cudaError_t hl_launch_compact_persist(const hl_compact_args *a, int nct, cudaStream_t s);
/* Tile masks of every image of a vote launch (nimg images: a->imgs, or
 * a->img0 when it is NULL); the vote kernel reads them. */
cudaError_t hl_launch_tile_masks(const hl_vote_args *a, int nimg,
                                 size_t max_words, cudaStream_t s);
/* words of an image's tile mask */
static inline size_t hl_tile_mask_words(int nslices, int nwin, int ntiles)
{
    return (size_t)nslices * nwin * ((ntiles + 31) / 32);
}
cudaError_t hl_launch_merge(const hl_merge_args *a, int max_rows, cudaStream_t s);
cudaError_t hl_launch_vote(const hl_vote_args *a, int threads, int grid,
                           cudaStream_t s);
size_t hl_vote_smem_bytes(int win_rows);
size_t hl_vote_points_smem_bytes(int win_rows);
cudaError_t hl_launch_vote_points(const int *xy, int n, const float *cosv,
                                  const float *sinv, int T, int Tp,
                                  int rho_min, int R, int win_rows, int nwin,
                                  float irho, int32_t *acc, int threads,
                                  cudaStream_t s);
cudaError_t hl_launch_peaks(const hl_peak_args *a, cudaStream_t s);
cudaError_t hl_launch_finalize(const hl_final_args *a, int nimg, cudaStream_t s);
cudaError_t hl_launch_to_tight(const int32_t *acc, int R, int T, int Tp,
                               int32_t *out, cudaStream_t s);
cudaError_t hl_launch_to_ref(const int32_t *acc, int R, int T, int Tp,
                             int rho_min, int ref_numrho, int32_t *ref,
                             cudaStream_t s);
cudaError_t hl_launch_from_tight(const int32_t *acc, int R, int T, int Tp,
                                 int32_t *out, cudaStream_t s);
cudaError_t hl_launch_bbox(const int *xy, int n, int *bbox, cudaStream_t s);
cudaError_t hl_launch_draw(uint8_t *out, long pitch, int w, int h,
                           const hl_line *lines, int nlines, int derho,
                           cudaStream_t s);
cudaError_t hl_launch_real_line(const uint8_t *img, long pitch, int w, int h,
                                int x1, int y1, int x2, int y2, int delta,
                                int *count, cudaStream_t s);
cudaError_t hl_launch_atomic_bench(int iters, int *sink, cudaStream_t s,
                                   int *blocks_out, int *threads_out);

#endif
