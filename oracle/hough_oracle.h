/*
 * hough_oracle.h -- CPU restatement of OpenCUDA's plain HoughLine path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * implementation in opencuda_gb300/: only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it.  The product never calls it.
 *
 * Every function cites the reference lines it restates (paths are relative to
 * the OpenCUDA project root, okano_3_0/ = the library directory).
 *
 * Accumulator layout used here ("tight layout"): acc[row * T + k], int32,
 * row = rho_bin - rho_min, 0 <= row < R, 0 <= k < T (rho-major, theta
 * contiguous -- the reference's own order without its one-bin zero border).
 *
 * Parity pinning: the vote rule is pinned against the reference kernel
 * _houghlineImgKer run on a GB300 (golden hashes in tests/golden/); the
 * peak / rank / decode / merge tail is pinned by known-answer tests.
 */
#ifndef HOUGH_ORACLE_H
#define HOUGH_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* LineParam record: okano_3_0/HoughLine.h:70-74 */
typedef struct ho_line {
    float angle;
    int distance;
    int votes;
} ho_line;

/* numtheta = (int)(M_PI / detheta): okano_3_0/HoughLine.cu:671 */
int ho_numtheta(double detheta);

/* Reference accumulator height numrho = (int)((w + h) * 2 + 1) / derho,
 * okano_3_0/HoughLine.cu:670.  The reference row of rho bin r is
 * r + (numrho - 1) / 2. */
int ho_ref_numrho(int w, int h, double derho);

/* Tight rho layout for a w x h ROI: D = floor(sqrt(w^2 + h^2) / derho + 0.5),
 * rho bins [-D, D], R = 2D + 1.  512x512 -> 1449, 4096x4096 -> 11587. */
void ho_layout(int w, int h, double derho, int *rho_min, int *R);

/* theta_k = (float)(k * detheta) (okano_3_0/HoughLine.cu:115); cos/sin by the
 * host libm (cosf/sinf).  The parity tables come from the GPU instead; this
 * one is used only to report how many entries differ. */
void ho_trig_libm(int T, double detheta, float *cosv, float *sinv);

/* Vote rule of _houghlineImgKer, okano_3_0/HoughLine.cu:86-130:
 *   pixel (c, r) of the ROI votes iff value == 255;
 *   for k in [0, T): rho = trunc(fl(fl(c * cos_k) * irho) + fl(fl(r * sin_k) * irho))
 * (the +-0.5 step at :121 is a no-op on an integer-valued float).
 * For derho == 1 the multiply by irho is exact and is skipped.
 * acc (R*T int32) is ADDED to (caller zeroes).  Returns the number of votes
 * whose bin fell outside [rho_min, rho_min + R) (always 0 for the tight
 * layout; counted, never written).  nthreads <= 0 -> all OpenMP threads. */
long long ho_vote_image(const uint8_t *roi, long pitch, int w, int h,
                        const float *cosv, const float *sinv, int T,
                        double derho, int rho_min, int R, int32_t *acc,
                        int nthreads);

/* Same rule over an interleaved (x, y) int coordinate list,
 * _houghlineCorKer, okano_3_0/HoughLine.cu:133-165. */
long long ho_vote_points(const int *xy, long n,
                         const float *cosv, const float *sinv, int T,
                         double derho, int rho_min, int R, int32_t *acc,
                         int nthreads);

/* Bounds-checked peak rule of _findlocalMaxKer, okano_3_0/HoughLine.cu:168-213:
 *   v > thr && v > acc[k-1] && v >= acc[k+1] && v > acc[row-1] && v >= acc[row+1]
 * with zero outside the grid (no theta wrap-around).  Writes the tight index
 * row*T+k of each peak in raster order (okano_3_0/HoughLine.cu:837-848) and
 * returns the total count (writes at most cap). */
long ho_peaks(const int32_t *acc, int R, int T, int thr,
              int32_t *idx_out, long cap);

/* Ranking modes for ho_rank_merge. */
#define HO_RANK_CANONICAL 0   /* votes desc, then raster index asc */
#define HO_RANK_REF_SHELL 1   /* the reference's unstable Shell sort, :853-873 */

/* Scene geometry needed by the decode step. */
typedef struct ho_geom {
    int T;          /* numtheta */
    int rho_min;    /* tight layout */
    int R;
    int ref_numrho; /* ho_ref_numrho(...) */
    double detheta;
    int thresdis;
    float thresang;
} ho_geom;

/* Host tail, okano_3_0/HoughLine.cu:853-948: rank the peaks, decode each
 * reference index (float scale decode, :884-897, including its +1 on negative
 * rho bins), greedy merge (:900-927), truncate to *linesmax (:932-948).
 * idx[] are tight indices of peaks (any order), votes looked up in acc.
 * On return *linesmax = min(survivors, *linesmax) and lines[0..*linesmax)
 * are written.  Returns the total survivor count (linenum). */
int ho_rank_merge(const int32_t *acc, const ho_geom *g,
                  const int32_t *idx, long n, int mode,
                  int *linesmax, ho_line *lines);

/* Convert a reference index to (row in tight layout, k) with the reference's
 * float decode; exposed for tests. */
void ho_decode_ref(const ho_geom *g, int ref_idx, int *tight_row, int *k,
                   float *angle, int *distance);

/* Tight -> reference layout: ref[(row_ref + 1) * (T + 2) + k + 1]
 * (okano_3_0/HoughLine.cu:124,683-705), ref zeroed first, size
 * (T + 2) * (ref_numrho + 2). */
void ho_to_ref_layout(const int32_t *acc, int R, int T, int rho_min,
                      int ref_numrho, int32_t *ref);

/* Whole plain pipeline on an ROI (vote -> peaks -> rank/merge); scratch is
 * allocated internally.  Returns linenum, or a negative value on failure. */
int ho_houghline_image(const uint8_t *roi, long pitch, int w, int h,
                       const float *cosv, const float *sinv,
                       double detheta, double derho, int threshold,
                       float thresang, int thresdis, int mode,
                       int *linesmax, ho_line *lines, int nthreads);

/* Line drawing of _houghoutKer, okano_3_0/HoughLine.cu:216-249: pixel (c, r)
 * of the w x h output is set to 255 if (int)(fl(c*cos(angle)) + fl(r*sin(angle)))
 * equals a line's distance (derho == 1).  cos/sin per line are supplied. */
void ho_draw_lines(uint8_t *out, long pitch, int w, int h,
                   const float *cosl, const float *sinl, const int *dist,
                   int nlines);

/* realLine's count, okano_3_0/HoughLine.cu:252-284 and :1377-1462: 255-pixels
 * of the w x h ROI inside the segment's box grown by delta = (int)threshold
 * whose distance |cross| / |segment| (double, stored as float) is below
 * delta.  Returns the count; *is_real = count > (int)|segment| * thresperc. */
int ho_real_line(const uint8_t *roi, long pitch, int w, int h, int x1, int y1,
                 int x2, int y2, float threshold, float thresperc,
                 int *is_real);

/* 64-bit FNV-1a of a byte range (fixture hashing). */
uint64_t ho_fnv1a(const void *p, size_t n);

int ho_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
