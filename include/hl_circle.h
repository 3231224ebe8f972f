/*
 * hl_circle.h -- HoughCircle on the GB300 HoughLine engine: C ABI.
 *
 * The image path of OpenCUDA's HoughCircle::houghcircle
 * (okano_3_0/HoughCircle.h:37-44, 226-235; okano_3_0/HoughCircle.cu:927-1214):
 * every 255-pixel of the ROI votes, for each radius in [radius_min,
 * radius_max], the points of the reference's midpoint circle into a
 * (radius, row, column) accumulator; local maxima above the threshold are
 * ranked by votes and merged greedily (centres closer than dist_thres and
 * radii closer than r_thres are averaged into the earlier circle); the first
 * *circlemax survivors are returned with the ROI offset added, as the
 * reference does.  Candidates with equal votes are ranked by their index
 * (radius, row, column) ascending: the reference's shear sort leaves their
 * order to its sorting network.
 */
#ifndef HL_CIRCLE_H
#define HL_CIRCLE_H

#include <stdint.h>

#include "houghline_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* CircleParam, okano_3_0/HoughCircle.h:37-44 */
typedef struct hl_circle {
    int a;        /* centre column */
    int b;        /* centre row */
    int radius;
    int votes;
} hl_circle;

/* HoughCircle's members (okano_3_0/HoughCircle.h:56-76; defaults 5, 50,
 * 50.0f, 20, 100): radius_min <= radius_max < 65536 */
typedef struct hl_circle_params {
    int radius_min, radius_max;
    float dist_thres;
    int r_thres;
    int threshold;
} hl_circle_params;

/* Circles of the image's ROI: *circlemax in (the room in out) / out (the
 * circles written).  Synchronises.  HL_OP_OVERFLOW when more than 4096
 * local maxima exceed the threshold (raise it). */
int hl_circles(hl_handle *h, const hl_image_desc *img, const hl_circle_params *p,
               int *circlemax, hl_circle *out, void *stream);

/* Circles of nimg ROIs (of one image or of several) in one pipeline: one
 * compaction, one tile launch and one tail launch for all of them, one copy of
 * the results.  counts[i] receives the circles of ROI i, written to
 * out[i * circlemax ..] (circlemax <= 4096); each ROI as hl_circles.  Returns
 * the first failing ROI's error (HL_OP_OVERFLOW: more than 4096 local maxima;
 * its count is 0); synchronises.  pieceCircle's pieces are one such call. */
int hl_circles_batch(hl_handle *h, const hl_image_desc *imgs, int nimg,
                     const hl_circle_params *p, int circlemax, hl_circle *out, int *counts,
                     void *stream);

/* The vote accumulator alone, for parity checks: acc_dev is a DEVICE array
 * of (radius_max - radius_min + 1) x roi_h x roi_w int32, [radius][row][col].
 * Synchronises (HL_CUDA_ERROR when a device-side wait gave up). */
int hl_circle_accumulator(hl_handle *h, const hl_image_desc *img,
                          const hl_circle_params *p, int32_t *acc_dev, void *stream);

#ifdef __cplusplus
}
#endif

#endif
