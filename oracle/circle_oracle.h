/*
 * circle_oracle.h -- CPU restatement of OpenCUDA's HoughCircle image path
 * (okano_3_0/HoughCircle.cu).  TEST INFRASTRUCTURE ONLY (see circle_oracle.c).
 */
#ifndef CIRCLE_ORACLE_H
#define CIRCLE_ORACLE_H

#include <stdint.h>

/* CircleParam, okano_3_0/HoughCircle.h:37-44 */
typedef struct hc_circle {
    int a, b, radius, votes;
} hc_circle;

/* acc[(z * h + y) * w + x], z = radius - rmin; returns the edge pixels */
long long hc_vote(const uint8_t *roi, long pitch, int w, int h, int rmin, int rmax,
                  int32_t *acc);
/* local maxima above threshold in (z, y, x) order; returns the count */
long hc_peaks(const int32_t *acc, int nr, int w, int h, int threshold, long *idx, long cap);
/* ranked, merged circles (ROI-local); *circlemax in/out; returns the
 * candidate count */
long hc_circles(const int32_t *acc, int nr, int w, int h, int rmin, int threshold,
                float dist_thres, int r_thres, int *circlemax, hc_circle *out);

#endif
