/*
 * circle_oracle.c -- CPU restatement of OpenCUDA's HoughCircle image path
 * (okano_3_0/HoughCircle.cu), TEST INFRASTRUCTURE ONLY: the GPU circle path
 * (opencuda_gb300/csrc/hl_circle.cu) is checked against it; nothing in the
 * product links or calls it.
 *
 * Parity: pinned by construction on the vote and peak rules and the merge
 * (each function below follows the cited reference lines); the reference's
 * own tests hold no golden vectors for this path.  One deliberate deviation,
 * shared with the GPU path: candidates with equal votes are ordered by their
 * raster index (radius, row, column) ascending, where the reference's shear
 * sort (okano_3_0/HoughCircle.cu:436-625, 765-800) leaves ties in an order
 * its 2-D sorting network happens to produce.
 */
#include "circle_oracle.h"

#include <stdlib.h>
#include <string.h>

/* one vote of the midpoint circle, okano_3_0/HoughCircle.cu:176-179 (the
 * VOTE macro: ROI-local coordinates, votes outside the ROI dropped) */
static void vote1(int32_t *acc, int w, int h, int x, int y, int z)
{
    if (x >= 0 && x < w && y >= 0 && y < h)
        acc[((size_t)z * h + y) * w + x] += 1;
}

/* okano_3_0/HoughCircle.cu:187-245 (_houghcirImgKer): every 255-pixel of the
 * ROI votes, for each radius rmin + z, the eight octant points of the
 * midpoint circle (x = 0, y = r, d = 3 - 2r; while x < y ...), the points on
 * the axes twice (x0 + 0 and x0 - 0 both vote). */
long long hc_vote(const uint8_t *roi, long pitch, int w, int h, int rmin, int rmax,
                  int32_t *acc)
{
    const int nr = rmax - rmin + 1;
    memset(acc, 0, sizeof(int32_t) * (size_t)nr * w * h);
    long long n = 0;
    for (int y0 = 0; y0 < h; y0++)
        for (int x0 = 0; x0 < w; x0++)
            n += roi[(size_t)y0 * pitch + x0] == 255;
    /* the radii are independent layers of the accumulator: one thread per
     * radius at a time, every pixel's votes for it in the reference order */
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < nr; z++) {
        const int radius = z + rmin;
        for (int y0 = 0; y0 < h; y0++)
            for (int x0 = 0; x0 < w; x0++) {
                if (roi[(size_t)y0 * pitch + x0] != 255)
                    continue;
                int x = 0, y = radius, d = 3 - 2 * radius;
                while (x < y) {
                    vote1(acc, w, h, x0 + x, y0 + y, z);
                    vote1(acc, w, h, x0 + x, y0 - y, z);
                    vote1(acc, w, h, x0 - x, y0 + y, z);
                    vote1(acc, w, h, x0 - x, y0 - y, z);
                    vote1(acc, w, h, x0 + y, y0 + x, z);
                    vote1(acc, w, h, x0 + y, y0 - x, z);
                    vote1(acc, w, h, x0 - y, y0 + x, z);
                    vote1(acc, w, h, x0 - y, y0 - x, z);
                    if (d < y)
                        d += 4 * x + 6;
                    else {
                        d += 4 * (x - y) + 10;
                        y--;
                    }
                    x++;
                }
            }
    }
    return n;
}

/* okano_3_0/HoughCircle.cu:321-370 (_findpartmaxKer) on the zero-bordered
 * slice of each radius, then the raster collection of :373-433: candidate
 * indices z*w*h + y*w + x in (z, y, x) order.  Returns the count (all of
 * them, even past cap; at most cap are stored). */
long hc_peaks(const int32_t *acc, int nr, int w, int h, int threshold, long *idx, long cap)
{
    long n = 0;
    for (int z = 0; z < nr; z++)
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) {
                const int32_t *p = acc + ((size_t)z * h + y) * w + x;
                const int v = p[0];
                const int L = x > 0 ? p[-1] : 0;
                const int R = x + 1 < w ? p[1] : 0;
                const int U = y > 0 ? p[-w] : 0;
                const int D = y + 1 < h ? p[w] : 0;
                if (v > threshold && v > L && v >= R && v > U && v >= D) {
                    if (n < cap)
                        idx[n] = ((long)z * h + y) * w + x;
                    n++;
                }
            }
    return n;
}

typedef struct { int votes; long idx; } hc_cand;

static int cand_cmp(const void *pa, const void *pb)
{
    const hc_cand *a = (const hc_cand *)pa, *b = (const hc_cand *)pb;
    if (a->votes != b->votes)
        return a->votes > b->votes ? -1 : 1;
    return a->idx < b->idx ? -1 : (a->idx > b->idx);
}

/* The tail: candidates ranked by votes (descending; ties by index), decoded
 * (okano_3_0/HoughCircle.cu:632-657: a = x, b = y, radius = z + rmin), merged
 * greedily (_recalCirParam, :809-871: a later circle whose centre lies
 * within dist_thres and whose radius within r_thres of the current one is
 * averaged into it -- integer halves -- and zeroed; the test is against the
 * current, already averaged, parameters and also meets zeroed circles; a
 * circle with zero votes or zero radius is passed over and not counted),
 * the first *circlemax survivors written.  Returns the candidate count. */
long hc_circles(const int32_t *acc, int nr, int w, int h, int rmin, int threshold,
                float dist_thres, int r_thres, int *circlemax, hc_circle *out)
{
    long n = hc_peaks(acc, nr, w, h, threshold, NULL, 0);
    if (n <= 0) {
        *circlemax = 0;
        return 0;
    }
    long *idx = (long *)malloc(sizeof(long) * (size_t)n);
    hc_cand *c = (hc_cand *)malloc(sizeof(hc_cand) * (size_t)n);
    hc_circle *cir = (hc_circle *)malloc(sizeof(hc_circle) * (size_t)n);
    hc_peaks(acc, nr, w, h, threshold, idx, n);
    for (long i = 0; i < n; i++) {
        c[i].idx = idx[i];
        c[i].votes = acc[idx[i]];
    }
    qsort(c, (size_t)n, sizeof(hc_cand), cand_cmp);
    const long size = (long)w * h;
    for (long i = 0; i < n; i++) {
        const long z = c[i].idx / size, t = c[i].idx - z * size;
        cir[i].a = (int)(t % w);
        cir[i].b = (int)(t / w);
        cir[i].radius = (int)z + rmin;
        cir[i].votes = c[i].votes;
    }
    int circlenum = 0;
    const float d2 = dist_thres * dist_thres;
    for (long i = 0; i < n; i++) {
        if (cir[i].votes == 0 || cir[i].radius == 0)
            continue;
        for (long j = i + 1; j < n; j++) {
            const int a1 = cir[i].a, b1 = cir[i].b, a2 = cir[j].a, b2 = cir[j].b;
            const int diffr = abs(cir[i].radius - cir[j].radius);
            const float distance = (float)(a1 - a2) * (a1 - a2) + (b1 - b2) * (b1 - b2);
            if (distance < d2 && diffr < r_thres) {
                cir[i].a = (cir[i].a + cir[j].a) / 2;
                cir[i].b = (cir[i].b + cir[j].b) / 2;
                cir[i].radius = (cir[i].radius + cir[j].radius) / 2;
                cir[i].votes = cir[i].votes + cir[j].votes;
                cir[j].a = cir[j].b = cir[j].radius = cir[j].votes = 0;
            }
        }
        circlenum++;
    }
    if (circlenum < *circlemax)
        *circlemax = circlenum;
    int k = 0;
    for (long i = 0; i < n && k < *circlemax; i++)
        if (cir[i].votes != 0)
            out[k++] = cir[i];
    free(idx);
    free(c);
    free(cir);
    return n;
}
