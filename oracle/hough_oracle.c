/*
 * hough_oracle.c -- CPU restatement of OpenCUDA's plain HoughLine path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  Build with
 * -O2 -ffp-contract=off so that every float operation is rounded exactly
 * as written; the CUDA kernels use __fmul_rn/__fadd_rn for the same reason.
 *
 * References are okano_3_0/HoughLine.cu (vote :86-130, coordinate vote
 * :133-165, peak :168-213, host tail :837-948, draw :216-249).
 */
#include "hough_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#error "glibc M_PI required: the reference's numtheta depends on it"
#endif

int ho_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* okano_3_0/HoughLine.cu:671 */
int ho_numtheta(double detheta)
{
    return (int)(M_PI / detheta);
}

/* okano_3_0/HoughLine.cu:670: int numrho = (int)((w + h) * 2 + 1) / derho; */
int ho_ref_numrho(int w, int h, double derho)
{
    return (int)((double)(int)((w + h) * 2 + 1) / derho);
}

void ho_layout(int w, int h, double derho, int *rho_min, int *R)
{
    double diag = sqrt((double)w * (double)w + (double)h * (double)h);
    int d = (int)floor(diag / derho + 0.5);
    *rho_min = -d;
    *R = 2 * d + 1;
}

void ho_trig_libm(int T, double detheta, float *cosv, float *sinv)
{
    for (int k = 0; k < T; k++) {
        float th = (float)(k * detheta);      /* okano_3_0/HoughLine.cu:115 */
        cosv[k] = cosf(th);
        sinv[k] = sinf(th);
    }
}

/* rho of one (x, y, k): okano_3_0/HoughLine.cu:117-121.  The cast to int
 * truncates toward zero; the following +-0.5 rounding of an integer-valued
 * float changes nothing, so it is not restated. */
static inline int rho_of(float x, float y, float c, float s, float irho,
                         int unit)
{
    float a = x * c;
    float b = y * s;
    if (!unit) {
        a = a * irho;
        b = b * irho;
    }
    return (int)(a + b);
}

long long ho_vote_image(const uint8_t *roi, long pitch, int w, int h,
                        const float *cosv, const float *sinv, int T,
                        double derho, int rho_min, int R, int32_t *acc,
                        int nthreads)
{
    /* The reference thread of pixel (c, r) loops over k (:111-127); the
     * order of the additions does not change an integer sum, so the edge
     * pixels (value == 255, :125) are listed once in raster order and the
     * theta columns are then voted in parallel. */
    long n = 0;
    for (int r = 0; r < h; r++)
        for (int col = 0; col < w; col++)
            n += (roi[(long)r * pitch + col] == 255);
    int *xy = (int *)malloc(sizeof(int) * 2 * (size_t)(n > 0 ? n : 1));
    if (!xy)
        return -1;
    long i = 0;
    for (int r = 0; r < h; r++) {
        const uint8_t *row = roi + (long)r * pitch;
        for (int col = 0; col < w; col++) {
            if (row[col] == 255) {
                xy[2 * i] = col;
                xy[2 * i + 1] = r;
                i++;
            }
        }
    }
    long long dropped = ho_vote_points(xy, n, cosv, sinv, T, derho, rho_min,
                                       R, acc, nthreads);
    free(xy);
    return dropped;
}

long long ho_vote_points(const int *xy, long n,
                         const float *cosv, const float *sinv, int T,
                         double derho, int rho_min, int R, int32_t *acc,
                         int nthreads)
{
    float irho = (float)(1.0 / derho);
    int unit = (derho == 1.0);
    long long dropped = 0;
    if (nthreads <= 0)
        nthreads = ho_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1) reduction(+:dropped)
    for (int k = 0; k < T; k++) {
        float c = cosv[k], s = sinv[k];
        for (long i = 0; i < n; i++) {
            int rho = rho_of((float)xy[2 * i], (float)xy[2 * i + 1], c, s,
                             irho, unit);            /* :143-160 */
            int bin = rho - rho_min;
            if (bin < 0 || bin >= R) {
                dropped++;
                continue;
            }
            acc[(long)bin * T + k] += 1;
        }
    }
    return dropped;
}

static inline int32_t at(const int32_t *acc, int R, int T, int row, int k)
{
    if (row < 0 || row >= R || k < 0 || k >= T)
        return 0;                 /* the reference's zero border */
    return acc[(long)row * T + k];
}

/* okano_3_0/HoughLine.cu:195-199 (peak test) and :837-848 (raster collect) */
long ho_peaks(const int32_t *acc, int R, int T, int thr,
              int32_t *idx_out, long cap)
{
    long n = 0;
    for (int row = 0; row < R; row++) {
        for (int k = 0; k < T; k++) {
            int32_t v = acc[(long)row * T + k];
            if (v > thr &&
                v > at(acc, R, T, row, k - 1) &&
                v >= at(acc, R, T, row, k + 1) &&
                v > at(acc, R, T, row - 1, k) &&
                v >= at(acc, R, T, row + 1, k)) {
                if (n < cap)
                    idx_out[n] = (int32_t)((long)row * T + k);
                n++;
            }
        }
    }
    return n;
}

/* Reference index of a tight bin: (row_ref + 1) * (T + 2) + k + 1 with
 * row_ref = rho + (numrho - 1) / 2 (okano_3_0/HoughLine.cu:122-124). */
static inline int ref_index(const ho_geom *g, int tight_idx)
{
    int row = tight_idx / g->T, k = tight_idx % g->T;
    int rho = row + g->rho_min;
    int row_ref = rho + (g->ref_numrho - 1) / 2;
    return (row_ref + 1) * (g->T + 2) + k + 1;
}

/* okano_3_0/HoughLine.cu:882-897 */
void ho_decode_ref(const ho_geom *g, int idx, int *tight_row, int *k,
                   float *angle, int *distance)
{
    float scale = (float)(1.0 / (g->T + 2));            /* :882-883 */
    int rho = (int)((float)idx * scale) - 1;             /* :886 */
    int theta = idx - (rho + 1) * (g->T + 2) - 1;        /* :888 */
    *angle = (float)(theta * g->detheta);                /* :889 */
    /* :891  rho - ((numrho-1)/2) - ((rho >= 0) ? -0.5f : 0.5f) */
    int rel = rho - ((g->ref_numrho - 1) / 2);
    float half = (rho >= 0) ? -0.5f : 0.5f;
    *distance = (int)((float)rel - half);
    if (tight_row)
        *tight_row = rel - g->rho_min;
    if (k)
        *k = theta;
}

typedef struct cand {
    int32_t votes;
    int32_t idx;    /* tight index */
} cand;

static int cmp_canonical(const void *a, const void *b)
{
    const cand *x = (const cand *)a, *y = (const cand *)b;
    if (x->votes != y->votes)
        return x->votes > y->votes ? -1 : 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

/* okano_3_0/HoughLine.cu:853-873, including its dead "j = j - gap". */
static void shell_sort_ref(cand *c, long sum)
{
    long gap = sum >> 1;
    while (gap > 0) {
        for (long i = gap; i < sum; i++) {
            cand t = c[i];
            long j = i - gap;
            while (j >= 0 && t.votes > c[j].votes) {
                c[j + gap] = c[j];
                j -= gap;
            }
            c[j + gap] = t;
        }
        gap >>= 1;
    }
}

/* The merge predicate of okano_3_0/HoughLine.cu:909-920. */
static inline int similar(const ho_line *a, const ho_line *b, int thresdis,
                          float thresang)
{
    float diffang = fabsf(a->angle - b->angle);
    int diffdis = abs(a->distance - b->distance);
    float diffang2 = (float)fabs(M_PI - (double)a->angle - (double)b->angle);
    int diffdis2 = abs(a->distance + b->distance);
    return (diffdis < thresdis && diffang < thresang) ||
           (diffdis2 < thresdis && diffang2 < thresang);
}

int ho_rank_merge(const int32_t *acc, const ho_geom *g,
                  const int32_t *idx, long n, int mode,
                  int *linesmax, ho_line *lines)
{
    cand *c = (cand *)malloc(sizeof(cand) * (size_t)(n > 0 ? n : 1));
    ho_line *line = (ho_line *)malloc(sizeof(ho_line) * (size_t)(n > 0 ? n : 1));
    if (!c || !line) {
        free(c);
        free(line);
        return -6;   /* OUT_OF_MEM */
    }
    for (long i = 0; i < n; i++) {
        c[i].idx = idx[i];
        c[i].votes = acc[idx[i]];
    }
    if (mode == HO_RANK_REF_SHELL)
        shell_sort_ref(c, n);
    else
        qsort(c, (size_t)n, sizeof(cand), cmp_canonical);

    for (long i = 0; i < n; i++) {                 /* :884-897 */
        int ri = ref_index(g, c[i].idx);
        ho_decode_ref(g, ri, NULL, NULL, &line[i].angle, &line[i].distance);
        line[i].votes = c[i].votes;
    }
    int linenum = 0;                               /* :900-927 */
    for (long i = 0; i < n; i++) {
        if (line[i].votes <= 0)
            continue;
        for (long j = i + 1; j < n; j++) {
            if (similar(&line[i], &line[j], g->thresdis, g->thresang)) {
                line[j].angle = 0.0f;
                line[j].distance = 0;
                line[j].votes = 0;
            }
        }
        linenum++;
    }
    *linesmax = (linenum < *linesmax) ? linenum : *linesmax;   /* :932 */
    int m = 0;                                     /* :935-948 */
    for (long i = 0; i < n && m < *linesmax; i++) {
        if (line[i].votes > 0)
            lines[m++] = line[i];
    }
    free(c);
    free(line);
    return linenum;
}

void ho_to_ref_layout(const int32_t *acc, int R, int T, int rho_min,
                      int ref_numrho, int32_t *ref)
{
    memset(ref, 0, sizeof(int32_t) * (size_t)(T + 2) * (size_t)(ref_numrho + 2));
    int off = (ref_numrho - 1) / 2;
    for (int row = 0; row < R; row++) {
        int row_ref = row + rho_min + off;
        if (row_ref < 0 || row_ref >= ref_numrho)
            continue;
        for (int k = 0; k < T; k++)
            ref[(long)(row_ref + 1) * (T + 2) + k + 1] = acc[(long)row * T + k];
    }
}

int ho_houghline_image(const uint8_t *roi, long pitch, int w, int h,
                       const float *cosv, const float *sinv,
                       double detheta, double derho, int threshold,
                       float thresang, int thresdis, int mode,
                       int *linesmax, ho_line *lines, int nthreads)
{
    ho_geom g;
    g.T = ho_numtheta(detheta);
    ho_layout(w, h, derho, &g.rho_min, &g.R);
    g.ref_numrho = ho_ref_numrho(w, h, derho);
    g.detheta = detheta;
    g.thresdis = thresdis;
    g.thresang = thresang;
    size_t bins = (size_t)g.R * (size_t)g.T;
    int32_t *acc = (int32_t *)calloc(bins, sizeof(int32_t));
    int32_t *pk = (int32_t *)malloc(sizeof(int32_t) * (bins / 2 + 2));
    if (!acc || !pk) {
        free(acc);
        free(pk);
        return -6;
    }
    ho_vote_image(roi, pitch, w, h, cosv, sinv, g.T, derho, g.rho_min, g.R,
                  acc, nthreads);
    long n = ho_peaks(acc, g.R, g.T, threshold, pk, (long)(bins / 2 + 2));
    int linenum = ho_rank_merge(acc, &g, pk, n, mode, linesmax, lines);
    free(acc);
    free(pk);
    return linenum;
}

/* okano_3_0/HoughLine.cu:216-249 with derho == 1. */
void ho_draw_lines(uint8_t *out, long pitch, int w, int h,
                   const float *cosl, const float *sinl, const int *dist,
                   int nlines)
{
    for (int r = 0; r < h; r++) {
        for (int c = 0; c < w; c++) {
            for (int i = 0; i < nlines; i++) {
                int t = (int)((float)c * cosl[i] + (float)r * sinl[i]);
                if (t == dist[i]) {
                    out[(long)r * pitch + c] = 255;
                    break;
                }
            }
        }
    }
}

int ho_real_line(const uint8_t *roi, long pitch, int w, int h, int x1, int y1,
                 int x2, int y2, float threshold, float thresperc,
                 int *is_real)
{
    int delta = (int)threshold;                 /* float -> int parameter */
    int xmax = x1 > x2 ? x1 : x2, xmin = x1 > x2 ? x2 : x1;
    int ymax = y1 > y2 ? y1 : y2, ymin = y1 > y2 ? y2 : y1;
    double len = sqrt((double)((x2 - x1) * (x2 - x1)) * 1.0 +
                      (double)((y2 - y1) * (y2 - y1)));
    int count = 0;
    for (int ry = 0; ry < h; ry++) {
        for (int cx = 0; cx < w; cx++) {
            if (!(cx <= xmax + delta && cx >= xmin - delta &&
                  ry <= ymax + delta && ry >= ymin - delta))
                continue;
            if (roi[(long)ry * pitch + cx] != 255)
                continue;
            int cr = abs((x2 - x1) * (ry - y1) - (cx - x1) * (y2 - y1));
            float dis = (float)((double)cr / len);
            if (dis < (float)delta)
                count++;
        }
    }
    int full = (int)sqrt(0.0 + (double)((x1 - x2) * (x1 - x2)) +
                         (double)((y1 - y2) * (y1 - y2)));   /* :1405 */
    if (is_real)
        *is_real = (float)count > (float)full * thresperc;
    return count;
}

uint64_t ho_fnv1a(const void *p, size_t n)
{
    const uint8_t *b = (const uint8_t *)p;
    uint64_t hsh = 1469598103934665603ull;
    for (size_t i = 0; i < n; i++) {
        hsh ^= b[i];
        hsh *= 1099511628211ull;
    }
    return hsh;
}
