/*
 * hl_api.cpp -- the C ABI: handle, workspace and the stage pipeline.
 *
 * hl_plain is HoughLine::houghLine (okano_3_0/HoughLine.cu:635-955) without
 * its per-call cudaMalloc/cudaFree and without the two accumulator-sized
 * device->host copies: four kernels run back to back on the caller's stream
 *   compact (a) -> vote (b) -> peaks (c1) -> finalize (c2)
 * and one small transfer brings back a header plus linesmax LineParam
 * records.  The workspace is owned by the handle and grows only when a
 * larger ROI arrives.
 */
#include <cuda_runtime.h>

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <queue>
#include <new>
#include <vector>

#include "hl_internal.h"
#include "hl_cnn.h"
#include "hl_proposal.h"
#include "hl_window.h"

#ifndef M_PI
#error "M_PI required: numtheta = (int)(M_PI / detheta)"
#endif

struct hl_batch_ws;   /* batched-path workspace (hl_batch*) */

struct hl_handle {
    hl_params p;
    int T, Tp;
    int device;
    int sms;
    float *d_cos, *d_sin;

    uint32_t *d_pts;
    size_t cap_pts;
    unsigned long long *d_tile_state;
    int *d_tile_off;
    size_t cap_tiles;
    int32_t *d_acc;
    size_t cap_acc;
    unsigned long long *d_keys;
    size_t cap_keys;
    int32_t *d_aux;          /* tight / reference layout staging */
    size_t cap_aux;
    unsigned char *d_result; /* hl_result_hdr + lines */
    size_t cap_result;
    unsigned char *h_result; /* pinned mirror */
    /* counters: [0] ncand, [1] status, [2] points, [3] ticket, [4..7] bbox */
    int *d_counters;

    unsigned ticket_base;
    unsigned epoch;
    int win_rows_override, threads_override;
    int last_launches;

    /* vote work items: heaviest-first order (cached per geometry) and the
     * persistent-CTA counter base */
    int4 *order_dev;
    size_t cap_order;
    int order_w, order_h, order_rows, order_R, order_T, order_ctas;
    int order_n, order_nmerge, order_nslots;
    /* the split blocks (summed from their parts' scratch slots) */
    hl_merge_region *d_merge;
    size_t cap_merge;
    int4 *d_scratch;
    size_t cap_scratch;
    /* HoughCircle: candidate keys, [ncand, status] counters, results; the
     * workspace of circle batches */
    struct hl_cb_ws *cb;
    unsigned long long *d_ckeys;
    int *d_ccnt;
    unsigned char *d_cres;
    unsigned char *h_cres;
    /* admitted-tile masks of the cached geometry (see hl_tile_mask_kernel) */
    unsigned *d_tmask;
    size_t cap_tmask;
    int masks_dirty;
    double order_detheta;
    double order_derho;
    unsigned work_base;

    /* batched path: workspace, CUDA-graph switch; whether the last
     * asynchronous call was a batch (hl_last_status reads its status) */
    hl_batch_ws *bw;
    hl_batch_ws *bw_fb;     /* the proposal path's fall-back batches */
    struct hl_prop_ws *pw;  /* the proposal path's own buffers */
    int batch_graph;
    int last_batch;

    /* per-stage CUDA-event timing (hl_profile) */
    int prof;
    int prof_open;
    int prof_used;
    cudaEvent_t *prof_ev;   /* HL_PROF_MAX x HL_NSTAGE+1 */
};

#define HL_NSTAGE 4
#define HL_PROF_MAX 512

/* Record the event that closes stage `st` (0 = before the first stage). */
static void prof_mark(hl_handle *h, int st, cudaStream_t s)
{
    if (!h->prof || !h->prof_ev || h->prof_used >= HL_PROF_MAX)
        return;
    if (st == 0)
        h->prof_open = 1;
    else if (!h->prof_open)
        return;   /* a call that did not start at stage (a) */
    cudaEventRecord(h->prof_ev[h->prof_used * (HL_NSTAGE + 1) + st], s);
    if (st == HL_NSTAGE) {
        h->prof_used++;
        h->prof_open = 0;
    }
}

static int map_err(cudaError_t e)
{
    if (e == cudaSuccess)
        return HL_NO_ERROR;
    if (e == cudaErrorMemoryAllocation)
        return HL_OUT_OF_MEM;
    return HL_CUDA_ERROR;
}

#define CK(call)                                  \
    do {                                          \
        cudaError_t e__ = (call);                 \
        if (e__ != cudaSuccess)                   \
            return map_err(e__);                  \
    } while (0)

static int grow(void **ptr, size_t *cap, size_t need_bytes)
{
    if (*cap >= need_bytes && *ptr)
        return HL_NO_ERROR;
    size_t nb = std::max(need_bytes, (size_t)256);
    nb = nb + nb / 4;   /* headroom for the next, slightly larger ROI */
    if (*ptr) {
        cudaFree(*ptr);   /* synchronises: nothing in flight uses it */
        *ptr = nullptr;
        *cap = 0;
    }
    cudaError_t e = cudaMalloc(ptr, nb);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return e == cudaErrorMemoryAllocation ? HL_OUT_OF_MEM : HL_CUDA_ERROR;
    }
    *cap = nb;
    return HL_NO_ERROR;
}

/* grow() that raises *moved when the buffer was (re)allocated */
static int grow_tracked(void **ptr, size_t *cap, size_t need_bytes, int *moved)
{
    const void *old = *ptr;
    int rc = grow(ptr, cap, need_bytes);
    if (rc == HL_NO_ERROR && *ptr != old)
        *moved = 1;
    return rc;
}

static int check_params(const hl_params *p)
{
    if (!(p->detheta > 0.0) || !(p->derho > 0.0))
        return HL_INVALID_DATA;
    double t = M_PI / p->detheta;
    if (!(t >= 1.0) || t > 65536.0)
        return HL_INVALID_DATA;
    return HL_NO_ERROR;
}

static int build_table(hl_handle *h)
{
    h->T = (int)(M_PI / h->p.detheta);          /* okano_3_0/HoughLine.cu:671 */
    h->Tp = (h->T + HL_SLICE - 1) / HL_SLICE * HL_SLICE;
    if (h->d_cos)
        cudaFree(h->d_cos);
    if (h->d_sin)
        cudaFree(h->d_sin);
    h->d_cos = h->d_sin = nullptr;
    CK(cudaMalloc(&h->d_cos, sizeof(float) * h->Tp));
    CK(cudaMalloc(&h->d_sin, sizeof(float) * h->Tp));
    CK(hl_launch_trig(h->d_cos, h->d_sin, h->T, h->Tp, h->p.detheta, 0));
    CK(cudaStreamSynchronize(0));
    return HL_NO_ERROR;
}

extern "C" int hl_create(hl_handle **out, const hl_params *params)
{
    if (!out)
        return HL_NULL_POINTER;
    *out = nullptr;
    hl_params p;
    if (params) {
        p = *params;
    } else {   /* okano_3_0/HoughLine.h:120-124 */
        p.detheta = M_PI / 180;
        p.derho = 1.0;
        p.threshold = 90;
        p.thresang = (float)(M_PI / 180 * 5.0f);
        p.thresdis = 50;
    }
    int rc = check_params(&p);
    if (rc != HL_NO_ERROR)
        return rc;
    hl_handle *h = new (std::nothrow) hl_handle();
    if (!h)
        return HL_OUT_OF_MEM;
    memset(h, 0, sizeof(*h));
    h->p = p;
    cudaError_t e = cudaGetDevice(&h->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount,
                                   h->device);
    if (e == cudaSuccess)
        e = cudaMalloc(&h->d_counters, 16 * sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemset(h->d_counters, 0, 16 * sizeof(int));
    if (e != cudaSuccess) {
        hl_destroy(h);
        return map_err(e);
    }
    rc = build_table(h);
    if (rc != HL_NO_ERROR) {
        hl_destroy(h);
        return rc;
    }
    *out = h;
    return HL_NO_ERROR;
}

static void batch_free(hl_handle *h);
static void circle_batch_free(hl_handle *h);

extern "C" int hl_destroy(hl_handle *h)
{
    if (!h)
        return HL_NULL_POINTER;
    batch_free(h);
    circle_batch_free(h);
    void *ptrs[] = {h->d_cos, h->d_sin, h->d_pts, h->d_tile_state,
                    h->d_tile_off, h->d_acc, h->d_keys, h->d_aux,
                    h->d_result, h->d_counters, h->order_dev,
                    h->d_merge, h->d_scratch, h->d_tmask,
                    h->d_ckeys, h->d_ccnt, h->d_cres};
    for (void *q : ptrs)
        if (q)
            cudaFree(q);
    if (h->h_result)
        cudaFreeHost(h->h_result);
    if (h->h_cres)
        cudaFreeHost(h->h_cres);
    if (h->prof_ev) {
        for (int i = 0; i < HL_PROF_MAX * (HL_NSTAGE + 1); i++)
            cudaEventDestroy(h->prof_ev[i]);
        free(h->prof_ev);
    }
    delete h;
    return HL_NO_ERROR;
}

extern "C" int hl_profile(hl_handle *h, int enable)
{
    if (!h)
        return HL_NULL_POINTER;
    if (enable && !h->prof_ev) {
        int n = HL_PROF_MAX * (HL_NSTAGE + 1);
        h->prof_ev = (cudaEvent_t *)calloc((size_t)n, sizeof(cudaEvent_t));
        if (!h->prof_ev)
            return HL_OUT_OF_MEM;
        for (int i = 0; i < n; i++)
            CK(cudaEventCreate(&h->prof_ev[i]));
    }
    h->prof = enable ? 1 : 0;
    h->prof_used = 0;
    return HL_NO_ERROR;
}

extern "C" int hl_profile_read(hl_handle *h, double *stage_ms, int *calls)
{
    if (!h || !stage_ms || !calls)
        return HL_NULL_POINTER;
    for (int s = 0; s < HL_NSTAGE; s++)
        stage_ms[s] = 0.0;
    *calls = h->prof_used;
    for (int c = 0; c < h->prof_used; c++) {
        cudaEvent_t *e = &h->prof_ev[c * (HL_NSTAGE + 1)];
        CK(cudaEventSynchronize(e[HL_NSTAGE]));
        for (int s = 0; s < HL_NSTAGE; s++) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, e[s], e[s + 1]));
            stage_ms[s] += ms;
        }
    }
    h->prof_used = 0;
    return HL_NO_ERROR;
}

extern "C" int hl_set_params(hl_handle *h, const hl_params *params)
{
    if (!h || !params)
        return HL_NULL_POINTER;
    int rc = check_params(params);
    if (rc != HL_NO_ERROR)
        return rc;
    bool retable = params->detheta != h->p.detheta;
    h->p = *params;
    return retable ? build_table(h) : HL_NO_ERROR;
}

extern "C" int hl_get_params(const hl_handle *h, hl_params *params)
{
    if (!h || !params)
        return HL_NULL_POINTER;
    *params = h->p;
    return HL_NO_ERROR;
}

static void layout(const hl_handle *h, double extent, int *rho_min, int *R)
{
    int d = (int)floor(extent / h->p.derho + 0.5);
    *rho_min = -d;
    *R = 2 * d + 1;
}

extern "C" int hl_geometry(const hl_handle *h, int w, int hh, hl_geom *g)
{
    if (!h || !g)
        return HL_NULL_POINTER;
    if (w <= 0 || hh <= 0 || w > HL_MAX_SIDE || hh > HL_MAX_SIDE)
        return HL_INVALID_DATA;
    g->numtheta = h->T;
    g->theta_pad = h->Tp;
    layout(h, sqrt((double)w * w + (double)hh * hh), &g->rho_min, &g->numrho);
    /* okano_3_0/HoughLine.cu:670 */
    g->ref_numrho = (int)((double)(int)((w + hh) * 2 + 1) / h->p.derho);
    g->tiles_x = (w + HL_TILE_W - 1) / HL_TILE_W;
    g->tiles_y = (hh + HL_TILE_H - 1) / HL_TILE_H;
    if ((double)g->numrho * h->Tp >= 2147483647.0)
        return HL_OP_OVERFLOW;
    return HL_NO_ERROR;
}

extern "C" int hl_trig_table(hl_handle *h, float *cos_host, float *sin_host)
{
    if (!h || !cos_host || !sin_host)
        return HL_NULL_POINTER;
    CK(cudaMemcpy(cos_host, h->d_cos, sizeof(float) * h->T,
                  cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(sin_host, h->d_sin, sizeof(float) * h->T,
                  cudaMemcpyDeviceToHost));
    return HL_NO_ERROR;
}

extern "C" int hl_set_vote_shape(hl_handle *h, int window_rows, int threads)
{
    if (!h)
        return HL_NULL_POINTER;
    if (window_rows < 0 || threads < 0 || threads > 1024 || (threads & 31))
        return HL_INVALID_DATA;
    if (window_rows > 65535 || (threads > 0 && threads < 64))
        return HL_INVALID_DATA;   /* rows above the shared-memory limit are clamped */
    h->win_rows_override = window_rows;
    h->threads_override = threads;
    return HL_NO_ERROR;
}

extern "C" int hl_last_launch_count(const hl_handle *h)
{
    return h ? h->last_launches : 0;
}

/* Rho-window rows per work item: at most what one CTA holds next to its
 * staging ring (one CTA of 1024 threads per SM), and enough windows that
 * there are about two items per SM (the heaviest-first order then balances
 * the tail), but no window below 256 rows. */
static void vote_shape(const hl_handle *h, int R, int *rows, int *nwin,
                       int *threads)
{
    const int slices = h->Tp / HL_SLICE;
    const int maxr = hl_vote_max_rows();
    int nw;
    if (h->win_rows_override > 0) {
        nw = (R + std::min(h->win_rows_override, maxr) - 1) /
             std::min(h->win_rows_override, maxr);
    } else {
        /* windows as tall as one CTA's shared memory allows (the fastest
         * measured at 4096 x 4096, T = 720: fewer tile-filter passes and
         * less vote waste than smaller windows; heavy blocks are split into
         * parts anyway), unless that leaves fewer blocks than SMs: then
         * about two blocks per SM, 256 rows at least */
        int nmin = (R + maxr - 1) / maxr;
        nw = nmin;
        if (nw * slices < std::max(h->sms, 1)) {
            int want = (2 * std::max(h->sms, 1) + slices - 1) / slices;
            int nmax = std::max(1, R / 256);
            nw = std::max(nmin, std::min(want, nmax));
        }
    }
    int r = (R + nw - 1) / nw;
    r = (r + 7) / 8 * 8;
    nw = (R + r - 1) / r;
    *rows = r;
    *nwin = nw;
    *threads = h->threads_override > 0 ? h->threads_override : 1024;
}

/* Weight of every (slice, window) block of a w x hh ROI: the area of the
 * tiles that the vote kernel's tile filter (tile_hits) admits for it.  The
 * kernel votes every point of an admitted tile with all 32 lanes (a last,
 * partial slice too: its lanes past T vote into the padding), so with a
 * uniform point density this is its work, waste included.  Per slice
 * each tile's rho range over the slice (corners at both end angles, plus
 * x + y when the corner's direction lies inside the slice, three bins of
 * slack) gives the run of windows it reaches. */
static void block_weights_tiles(const hl_handle *h, int w, int hh, int rho_min,
                                int R, int rows, int nwin,
                                std::vector<double> &wt)
{
    const int slices = h->Tp / HL_SLICE;
    const int tx_n = (w + HL_TILE_W - 1) / HL_TILE_W;
    const int ty_n = (hh + HL_TILE_H - 1) / HL_TILE_H;
    const double irho = 1.0 / h->p.derho;
    wt.assign((size_t)slices * nwin, 0.0);
    for (int sl = 0; sl < slices; sl++) {
        const int k0 = sl * HL_SLICE;
        if (k0 >= h->T)
            continue;
        const int k1 = std::min(k0 + HL_SLICE, h->T) - 1;
        const double c0 = cos(k0 * h->p.detheta), s0 = sin(k0 * h->p.detheta);
        const double c1 = cos(k1 * h->p.detheta), s1 = sin(k1 * h->p.detheta);
        for (int ty = 0; ty < ty_n; ty++) {
            const double ya = (double)ty * HL_TILE_H;
            const double yb = std::min(ya + HL_TILE_H - 1, hh - 1.0);
            for (int tx = 0; tx < tx_n; tx++) {
                const double xa = (double)tx * HL_TILE_W;
                const double xb = std::min(xa + HL_TILE_W - 1, w - 1.0);
                double mn = 1e300, mx = -1e300;
                for (int i = 0; i < 4; i++) {
                    const double x = (i & 1) ? xb : xa, y = (i & 2) ? yb : ya;
                    const double f0 = x * c0 + y * s0, f1 = x * c1 + y * s1;
                    mn = std::min(mn, std::min(f0, f1));
                    double hi = std::max(f0, f1);
                    if (c0 * y - s0 * x >= 0.0 && x * s1 - y * c1 >= 0.0)
                        hi = std::max(hi, x + y);
                    mx = std::max(mx, hi);
                }
                const double lo_r = mn * irho - 3.0 - rho_min;
                const double hi_r = mx * irho + 3.0 - rho_min;
                if (hi_r < 0.0 || lo_r > R - 1.0)
                    continue;
                int wlo = nwin > 1 ? (int)floor(std::max(lo_r, 0.0) / rows) : 0;
                int whi = nwin > 1 ? (int)floor(std::min(hi_r, R - 1.0) / rows) : 0;
                wlo = std::min(std::max(wlo, 0), nwin - 1);
                whi = std::min(std::max(whi, wlo), nwin - 1);
                const double area = (xb - xa + 1.0) * (yb - ya + 1.0);
                for (int wn = wlo; wn <= whi; wn++)
                    wt[(size_t)sl + (size_t)slices * wn] += area;
            }
        }
    }
}

/* Split plan of the vote blocks (weights wt in pixels of admitted tiles,
 * ctas persistent CTAs): a block heavier than cap = total / (capf * ctas) is
 * cut into ceil(wt / cap) parts (at most 16, none below HL_MIN_PART pixels:
 * a part's fixed cost -- its scratch slot, written and merged -- would
 * outweigh its votes).  Then one pass over a list schedule of the parts (each CTA
 * takes the next part, heaviest first, when it is free -- the vote kernel's
 * own order): a part that would start after 60% of the estimated makespan and
 * weighs more than cap / 4 is halved (part p of n becomes parts 2p and 2p + 1
 * of 2n, the same range of the block's batches), so the last parts to start
 * are small and the CTAs finish together.  Returns the parts heaviest first;
 * pieces[b] counts block b's parts. */
struct vote_part { double wt; int blk, part, nparts; };
#define HL_MIN_PART (256.0 * 1024.0)
static std::vector<vote_part> plan_parts(const std::vector<double> &wt, int ctas,
                                         double capf, std::vector<int> &pieces)
{
    double total = 0.0;
    for (double v : wt)
        total += v;
    const double cap = total / (capf * std::max(ctas, 1));
    std::vector<vote_part> parts;
    parts.reserve(wt.size() * 2);
    for (size_t b = 0; b < wt.size(); b++) {
        int np = 1;
        if (cap > 0.0 && wt[b] > cap)
            np = std::min(16, (int)ceil(wt[b] / cap));
        np = std::max(1, std::min(np, (int)(wt[b] / HL_MIN_PART)));
        for (int q = 0; q < np; q++)
            parts.push_back({wt[b] / np, (int)b, q, np});
    }
    const auto heavier = [](const vote_part &a, const vote_part &c) { return a.wt > c.wt; };
    std::stable_sort(parts.begin(), parts.end(), heavier);
    {
        typedef std::pair<double, int> slot_t;
        std::priority_queue<slot_t, std::vector<slot_t>, std::greater<slot_t>> free_at;
        for (int c = 0; c < std::max(ctas, 1); c++)
            free_at.push({0.0, c});
        std::vector<double> start(parts.size());
        double makespan = 0.0;
        for (size_t i = 0; i < parts.size(); i++) {
            slot_t f = free_at.top();
            free_at.pop();
            start[i] = f.first;
            makespan = std::max(makespan, f.first + parts[i].wt);
            free_at.push({f.first + parts[i].wt, f.second});
        }
        std::vector<vote_part> out;
        out.reserve(parts.size() * 2);
        for (size_t i = 0; i < parts.size(); i++) {
            const vote_part &p = parts[i];
            if (start[i] > 0.6 * makespan && p.wt > 0.25 * cap && p.nparts <= 16 &&
                p.wt >= 2.0 * HL_MIN_PART) {
                out.push_back({p.wt / 2, p.blk, 2 * p.part, 2 * p.nparts});
                out.push_back({p.wt / 2, p.blk, 2 * p.part + 1, 2 * p.nparts});
            } else {
                out.push_back(p);
            }
        }
        parts.swap(out);
    }
    std::stable_sort(parts.begin(), parts.end(), heavier);
    pieces.assign(wt.size(), 0);
    for (const vote_part &p : parts)
        pieces[p.blk]++;
    return parts;
}

/* Work items of the vote kernel, heaviest first, weighted by
 * block_weights_tiles.  A block heavier than half of one CTA's fair share
 * (total / ctas; a third and a quarter measured slower at 4096 x 4096) is
 * split into parts that each vote a contiguous share of the point stream
 * (at most 16 parts), each voting into its own scratch slot; the merge
 * launch after the vote sums a split block's slots.  Cached per geometry with
 * the list of split blocks; fills va's items and scratch. */
static int vote_items(hl_handle *h, int w, int hh, int rho_min, int R,
                      int rows, int nwin, int ctas, hl_vote_args *va)
{
    const int slices = h->Tp / HL_SLICE;
    const int nblocks = slices * nwin;
    if (!(h->order_dev && h->order_w == w && h->order_h == hh &&
          h->order_rows == rows && h->order_R == R && h->order_T == h->T &&
          h->order_derho == h->p.derho && h->order_detheta == h->p.detheta &&
          h->order_ctas == ctas)) {
        h->masks_dirty = 1;
        std::vector<double> wt;
        block_weights_tiles(h, w, hh, rho_min, R, rows, nwin, wt);
        std::vector<int> pieces;
        const std::vector<vote_part> parts = plan_parts(wt, ctas, 2.0, pieces);
        /* scratch slots and merge regions of the split blocks */
        std::vector<hl_merge_region> merge;
        std::vector<int> slot0((size_t)nblocks, 0), used((size_t)nblocks, 0);
        int nslots = 0;
        for (int b = 0; b < nblocks; b++) {
            if (pieces[b] <= 1)
                continue;
            const int w0 = (b / slices) * rows, k0 = (b % slices) * HL_SLICE;
            const long long off = (long long)w0 * h->Tp + k0;
            slot0[b] = nslots;
            merge.push_back({off / 4, std::min(rows, R - w0), k0, nslots, pieces[b], w0, 0, {0, 0}});
            nslots += pieces[b];
        }
        const int n = (int)parts.size();
        std::vector<int4> items((size_t)n);
        for (int i = 0; i < n; i++) {
            const vote_part &p = parts[i];
            const int slot = pieces[p.blk] > 1 ? slot0[p.blk] + used[p.blk]++ : 0;
            items[i] = make_int4(p.blk, p.part | (p.nparts << 16), slot, 0);
        }
        int rc = grow((void **)&h->order_dev, &h->cap_order, sizeof(int4) * (size_t)n);
        if (rc == HL_NO_ERROR && !merge.empty())
            rc = grow((void **)&h->d_merge, &h->cap_merge,
                      sizeof(hl_merge_region) * merge.size());
        if (rc != HL_NO_ERROR)
            return rc;
        CK(cudaMemcpy(h->order_dev, items.data(), sizeof(int4) * (size_t)n,
                      cudaMemcpyHostToDevice));
        if (!merge.empty())
            CK(cudaMemcpy(h->d_merge, merge.data(), sizeof(hl_merge_region) * merge.size(),
                          cudaMemcpyHostToDevice));
        h->order_w = w;
        h->order_h = hh;
        h->order_rows = rows;
        h->order_R = R;
        h->order_T = h->T;
        h->order_derho = h->p.derho;
        h->order_detheta = h->p.detheta;
        h->order_ctas = ctas;
        h->order_n = n;
        h->order_nmerge = (int)merge.size();
        h->order_nslots = nslots;
    }
    int rc = grow((void **)&h->d_scratch, &h->cap_scratch,
                  sizeof(int4) * (size_t)std::max(h->order_nslots, 1) * rows * (HL_SLICE / 4));
    if (rc != HL_NO_ERROR)
        return rc;
    va->items = h->order_dev;
    va->nitems = h->order_n;
    va->scratch = h->d_scratch;
    return HL_NO_ERROR;
}

static int ensure_image(hl_handle *h, const hl_geom &g, int w, int hh)
{
    int rc;
    size_t ntiles = (size_t)g.tiles_x * g.tiles_y;
    if ((rc = grow((void **)&h->d_pts, &h->cap_pts,
                   sizeof(float2) * ((size_t)w * hh + 16))) != HL_NO_ERROR)
        return rc;
    if (h->cap_tiles < ntiles + 1 || !h->d_tile_state) {
        size_t cap = 0;
        if ((rc = grow((void **)&h->d_tile_state, &cap,
                       sizeof(unsigned long long) * (ntiles + 1))) != HL_NO_ERROR)
            return rc;
        CK(cudaMemset(h->d_tile_state, 0, cap));
        size_t cap2 = 0;
        if ((rc = grow((void **)&h->d_tile_off, &cap2,
                       sizeof(int) * (ntiles + 1))) != HL_NO_ERROR)
            return rc;
        h->cap_tiles = std::min(cap / sizeof(unsigned long long),
                                cap2 / sizeof(int));
    }
    return HL_NO_ERROR;
}

/* Peak candidates (batches): the list and its room; a threshold that only
 * peaks-to-be clear leaves a few hundred per image, and past the room the
 * peak pass scans the accumulators instead.  A null list: no noting. */
static hl_cand_list cand_list(unsigned long long *e, size_t cap_bytes, int *count)
{
    hl_cand_list c;
    c.e = e;
    c.count = count;
    c.cap = (int)std::min(cap_bytes / sizeof(unsigned long long), (size_t)0x7fffffff);
    c.pad = 0;
    return c;
}

static int ensure_acc(hl_handle *h, int R, int linesmax)
{
    int rc;
    size_t bins = (size_t)R * h->Tp;
    if ((rc = grow((void **)&h->d_acc, &h->cap_acc, sizeof(int32_t) * bins)) !=
        HL_NO_ERROR)
        return rc;
    /* peaks never sit next to each other along theta: at most ceil(T/2)
     * per rho row */
    size_t maxpk = (size_t)R * ((h->T + 1) / 2) + 32;
    if ((rc = grow((void **)&h->d_keys, &h->cap_keys,
                   sizeof(unsigned long long) * maxpk)) != HL_NO_ERROR)
        return rc;
    size_t lm = (size_t)std::max(linesmax, 1);
    size_t rbytes = sizeof(hl_result_hdr) + sizeof(hl_line) * lm;
    if (h->cap_result < rbytes || !h->d_result) {
        if ((rc = grow((void **)&h->d_result, &h->cap_result, rbytes)) !=
            HL_NO_ERROR)
            return rc;
        if (h->h_result)
            cudaFreeHost(h->h_result);
        h->h_result = nullptr;
        CK(cudaMallocHost(&h->h_result, h->cap_result));
    }
    return HL_NO_ERROR;
}

static int key_cap(const hl_handle *h)
{
    size_t c = h->cap_keys / sizeof(unsigned long long);
    return (int)std::min(c, (size_t)0x7fffffff);
}

static int roi_of(const hl_image_desc *img, hl_roi *roi)
{
    if (!img || !img->data)
        return HL_NULL_POINTER;
    /* okano_3_0/Image.h:218-258: the ROI must lie inside the image */
    if (img->width <= 0 || img->height <= 0 || img->pitch < (size_t)img->width)
        return HL_INVALID_DATA;
    if (img->roi_x1 < 0 || img->roi_y1 < 0 || img->roi_x2 > img->width ||
        img->roi_y2 > img->height || img->roi_x2 <= img->roi_x1 ||
        img->roi_y2 <= img->roi_y1)
        return HL_INVALID_DATA;
    roi->w = img->roi_x2 - img->roi_x1;
    roi->h = img->roi_y2 - img->roi_y1;
    if (roi->w > HL_MAX_SIDE || roi->h > HL_MAX_SIDE)
        return HL_INVALID_DATA;
    roi->base = img->data + (size_t)img->roi_y1 * img->pitch + img->roi_x1;
    roi->pitch = (long)img->pitch;
    return HL_NO_ERROR;
}

/* stages (a) + (b) into h->d_acc ([R][Tp]) */
/* Stage (a) of one image's ROI into h->d_pts (float2, tile-major, odd tiles
 * padded), h->d_tile_off and the point count h->d_counters[2]: about one
 * CTA per SM when they fit at once, else one CTA per 4-tile group. */
static int launch_compaction(hl_handle *h, const hl_roi &roi, const hl_geom &g,
                             cudaStream_t s)
{
    const int ntiles = g.tiles_x * g.tiles_y;
    hl_compact_args ca;
    memset(&ca, 0, sizeof(ca));
    ca.roi = roi;
    ca.tiles_x = g.tiles_x;
    ca.ntiles = ntiles;
    ca.tile_state = h->d_tile_state;
    ca.ticket = reinterpret_cast<unsigned *>(h->d_counters + 3);
    ca.ticket_base = h->ticket_base;
    if (++h->epoch >= (1u << 30)) {
        CK(cudaMemsetAsync(h->d_tile_state, 0,
                           sizeof(unsigned long long) * h->cap_tiles, s));
        h->epoch = 1;
    }
    ca.epoch = h->epoch;
    ca.pts = nullptr;
    ca.pts_f2 = reinterpret_cast<float2 *>(h->d_pts);
    ca.tile_off = h->d_tile_off;
    ca.count = h->d_counters + 2;
    ca.status = h->d_counters + 1;
    const int nct = hl_compact_persist_ctas(ntiles, h->sms);
    if (nct > 0) {
        CK(hl_launch_compact_persist(&ca, nct, s));
        h->ticket_base += (unsigned)nct;
    } else {
        CK(hl_launch_compact(&ca, s));
        h->ticket_base += (unsigned)((ntiles + HL_COMPACT_GROUP - 1) / HL_COMPACT_GROUP);
    }
    return HL_NO_ERROR;
}

static int run_ab(hl_handle *h, const hl_roi &roi, const hl_geom &g,
                  cudaStream_t s, int *launches)
{
    const int ntiles = g.tiles_x * g.tiles_y;

    /* the vote plan first: its split blocks' regions are cleared by the
     * compaction launch, and its tile masks are computed once per geometry */
    hl_vote_args va;
    memset(&va, 0, sizeof(va));
    va.imgs = nullptr;
    va.img0.pts = reinterpret_cast<const float2 *>(h->d_pts);
    va.img0.tile_off = h->d_tile_off;
    va.img0.ntiles = ntiles;
    va.img0.tiles_x = g.tiles_x;
    va.img0.w = roi.w;
    va.img0.h = roi.h;
    va.img0.rho_min = g.rho_min;
    va.img0.R = g.numrho;
    va.img0.threshold = h->p.threshold;
    va.img0.acc = h->d_acc;
    va.cosv = h->d_cos;
    va.sinv = h->d_sin;
    va.T = h->T;
    va.Tp = h->Tp;
    int threads;
    vote_shape(h, g.numrho, &va.win_rows, &va.img0.nwin, &threads);
    va.irho = (float)(1.0 / h->p.derho);   /* okano_3_0/HoughLine.cu:107 */
    va.status = h->d_counters + 1;
    va.part16 = hl_part16_ok(h->p.derho, roi.w, roi.h);
    /* one image: no candidate list (the peak pass scans the accumulator,
     * which is still in L2; noting measured slower on the whole step) */
    va.cand = cand_list(nullptr, 0, nullptr);
    /* persistent CTAs: as many as fit (one per SM at 1024 threads) */
    const size_t smem = hl_vote_smem_bytes(va.win_rows);
    const int per_sm = std::max(1, std::min(2048 / threads,
                                            (int)((228u * 1024u) / (smem + 1024))));
    const int ctas = std::max(h->sms, 1) * per_sm;
    int rc = vote_items(h, roi.w, roi.h, g.rho_min, g.numrho, va.win_rows,
                        va.img0.nwin, ctas, &va);
    if (rc != HL_NO_ERROR)
        return rc;
    const size_t mwords = hl_tile_mask_words(h->Tp / HL_SLICE, va.img0.nwin, ntiles);
    const void *old_mask = h->d_tmask;
    if ((rc = grow((void **)&h->d_tmask, &h->cap_tmask, sizeof(unsigned) * mwords)) !=
        HL_NO_ERROR)
        return rc;
    if (h->d_tmask != old_mask)
        h->masks_dirty = 1;
    va.img0.tmask = h->d_tmask;
    if (h->masks_dirty) {
        CK(hl_launch_tile_masks(&va, 1, mwords, s));
        (*launches)++;
        h->masks_dirty = 0;
    }

    prof_mark(h, 0, s);
    rc = launch_compaction(h, roi, g, s);
    if (rc != HL_NO_ERROR)
        return rc;
    (*launches)++;
    prof_mark(h, 1, s);

    const int grid = std::min(va.nitems, ctas);
    va.work = reinterpret_cast<unsigned *>(h->d_counters + 9);
    va.work_base = h->work_base;
    CK(hl_launch_vote(&va, threads, grid, s));
    /* every CTA takes one ticket per item plus one that finds no item */
    h->work_base += (unsigned)(va.nitems + grid);
    (*launches)++;
    if (h->order_nmerge > 0) {
        hl_merge_args ma;
        ma.acc = reinterpret_cast<int4 *>(h->d_acc);
        ma.pitch4 = h->Tp / 4;
        ma.T = h->T;
        ma.scratch = h->d_scratch;
        ma.slot4 = hl_slot4(va.win_rows, va.part16);
        ma.regs = h->d_merge;
        ma.nreg = h->order_nmerge;
        ma.part16 = va.part16;
        ma.pimgs = nullptr;
        ma.thr0 = h->p.threshold;
        ma.cand = va.cand;
        CK(hl_launch_merge(&ma, va.win_rows, s));
        (*launches)++;
    }
    prof_mark(h, 2, s);
    return HL_NO_ERROR;
}

/* stage (c) over h->d_acc */
/* the tail's arguments for one image: the handle's keys and counters, the
 * result records into lines_dev (or the handle's result buffer) */
static void final_args(hl_handle *h, const hl_geom &g, int linesmax, hl_line *lines_dev,
                       int *count_dev, hl_final_args *fa)
{
    memset(fa, 0, sizeof(*fa));
    fa->imgs = nullptr;
    fa->img0.keys = h->d_keys;
    fa->img0.ncand = h->d_counters + 0;
    fa->img0.cap = key_cap(h);
    fa->img0.rho_min = g.rho_min;
    fa->img0.ref_numrho = g.ref_numrho;
    fa->img0.pad = 0;
    fa->T = h->T;
    fa->detheta = h->p.detheta;
    fa->thresdis = h->p.thresdis;
    fa->thresang = h->p.thresang;
    fa->linesmax = linesmax;
    fa->hdr = reinterpret_cast<hl_result_hdr *>(h->d_result);
    fa->img0.lines = lines_dev ? lines_dev
                               : reinterpret_cast<hl_line *>(h->d_result +
                                                             sizeof(hl_result_hdr));
    fa->status = h->d_counters + 1;
    fa->img0.count_out = count_dev;
}

static int run_c(hl_handle *h, const hl_geom &g, int linesmax,
                 hl_line *lines_dev, int *count_dev, cudaStream_t s,
                 int *launches)
{
    hl_peak_args pa;
    pa.imgs = nullptr;
    pa.img0.acc = h->d_acc;
    pa.img0.keys = h->d_keys;
    pa.img0.ncand = h->d_counters + 0;
    pa.img0.R = g.numrho;
    pa.img0.cap = key_cap(h);
    pa.img0.threshold = h->p.threshold;
    pa.img0.pad = 0;
    pa.chunks = nullptr;
    /* units of HL_PEAK_FLAT int4; the kernel indexes the accumulator's int4
     * in 32 bits */
    if ((long long)g.numrho * (h->Tp / 4) >= (1LL << 32))
        return HL_OP_OVERFLOW;
    pa.nchunks = (int)(((long long)g.numrho * (h->Tp / 4) + HL_PEAK_FLAT - 1) / HL_PEAK_FLAT);
    pa.T = h->T;
    pa.Tp = h->Tp;
    pa.status = h->d_counters + 1;
    pa.cand = cand_list(nullptr, 0, nullptr);
    CK(hl_launch_peaks(&pa, s));
    (*launches)++;
    prof_mark(h, 3, s);

    hl_final_args fa;
    final_args(h, g, linesmax, lines_dev, count_dev, &fa);
    CK(hl_launch_finalize(&fa, 1, s));
    (*launches)++;
    prof_mark(h, 4, s);
    return HL_NO_ERROR;
}

/* After a device-side failure the ticket / work counters may not have
 * advanced by what the host expects: zero them and their bases. */
static void reset_counters(hl_handle *h, cudaStream_t s)
{
    cudaMemsetAsync(h->d_counters, 0, 16 * sizeof(int), s);
    cudaStreamSynchronize(s);
    h->ticket_base = 0;
    h->work_base = 0;
}

static int fetch_result(hl_handle *h, int *linesmax, hl_line *lines,
                        cudaStream_t s)
{
    int lm = std::max(*linesmax, 0);
    size_t bytes = sizeof(hl_result_hdr) + sizeof(hl_line) * (size_t)lm;
    CK(cudaMemcpyAsync(h->h_result, h->d_result, bytes, cudaMemcpyDeviceToHost,
                       s));
    CK(cudaStreamSynchronize(s));
    const hl_result_hdr *hdr = reinterpret_cast<const hl_result_hdr *>(h->h_result);
    if (hdr->status != 0) {
        reset_counters(h, s);
        return HL_CUDA_ERROR;
    }
    int cnt = hdr->count;
    if (cnt > 0 && lines)
        memcpy(lines, h->h_result + sizeof(hl_result_hdr),
               sizeof(hl_line) * (size_t)cnt);
    *linesmax = cnt;
    return HL_NO_ERROR;
}

static int plain_launch(hl_handle *h, const hl_image_desc *img, int linesmax,
                        hl_line *lines_dev, int *count_dev, cudaStream_t s,
                        int ref_numrho_override = 0)
{
    hl_roi roi;
    int rc = roi_of(img, &roi);
    if (rc != HL_NO_ERROR)
        return rc;
    hl_geom g;
    if ((rc = hl_geometry(h, roi.w, roi.h, &g)) != HL_NO_ERROR)
        return rc;
    if (ref_numrho_override > 0)
        g.ref_numrho = ref_numrho_override;
    if ((rc = ensure_image(h, g, roi.w, roi.h)) != HL_NO_ERROR)
        return rc;
    if ((rc = ensure_acc(h, g.numrho, linesmax)) != HL_NO_ERROR)
        return rc;
    int launches = 0;
    h->last_batch = 0;
    if (!h->win_rows_override && !h->threads_override && !h->prof &&
        hl_small_fits(h->T, h->Tp, g.numrho)) {
        /* a small image: the whole path in one cluster launch, the
         * accumulator in shared memory only */
        hl_small_args sa;
        memset(&sa, 0, sizeof(sa));
        sa.roi = roi;
        sa.pts = reinterpret_cast<float2 *>(h->d_pts);
        sa.cosv = h->d_cos;
        sa.sinv = h->d_sin;
        sa.T = h->T;
        sa.Tp = h->Tp;
        sa.R = g.numrho;
        sa.rho_min = g.rho_min;
        sa.irho = (float)(1.0 / h->p.derho);   /* okano_3_0/HoughLine.cu:107 */
        sa.threshold = h->p.threshold;
        final_args(h, g, linesmax, lines_dev, count_dev, &sa.fin);
        sa.scale = (float)(1.0 / (h->T + 2));  /* :882-883 */
        CK(hl_launch_small(&sa, s));
        h->last_launches = 1;
        return HL_NO_ERROR;
    }
    if ((rc = run_ab(h, roi, g, s, &launches)) != HL_NO_ERROR)
        return rc;
    rc = run_c(h, g, linesmax, lines_dev, count_dev, s, &launches);
    h->last_launches = launches;
    return rc;
}

extern "C" int hl_plain(hl_handle *h, const hl_image_desc *img, int *linesmax,
                        hl_line *lines, void *stream)
{
    if (!h || !img || !linesmax)
        return HL_NULL_POINTER;
    if (*linesmax > 0 && !lines)
        return HL_NULL_POINTER;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int rc = plain_launch(h, img, *linesmax, nullptr, nullptr, s);
    if (rc != HL_NO_ERROR)
        return rc;
    return fetch_result(h, linesmax, lines, s);
}

extern "C" int hl_plain_async(hl_handle *h, const hl_image_desc *img,
                              int linesmax, hl_line *lines_dev, int *count_dev,
                              void *stream)
{
    if (!h || !img)
        return HL_NULL_POINTER;
    if (linesmax > 0 && !lines_dev)
        return HL_NULL_POINTER;
    return plain_launch(h, img, linesmax, lines_dev, count_dev,
                        reinterpret_cast<cudaStream_t>(stream));
}

static int batch_last_status(hl_handle *h, int *status, cudaStream_t s);

extern "C" int hl_last_status(hl_handle *h, int *status, void *stream)
{
    if (!h || !status)
        return HL_NULL_POINTER;
    hl_result_hdr hdr;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (h->last_batch)
        return batch_last_status(h, status, s);
    if (!h->d_result) {
        *status = 0;
        return HL_NO_ERROR;
    }
    CK(cudaMemcpyAsync(&hdr, h->d_result, sizeof(hdr), cudaMemcpyDeviceToHost,
                       s));
    CK(cudaStreamSynchronize(s));
    *status = hdr.status;
    if (hdr.status != 0)
        reset_counters(h, s);
    return HL_NO_ERROR;
}

extern "C" int hl_compact(hl_handle *h, const hl_image_desc *img,
                          uint32_t *pts_dev, int *tile_off_dev, int *count_dev,
                          void *stream)
{
    if (!h || !img || !pts_dev || !tile_off_dev || !count_dev)
        return HL_NULL_POINTER;
    hl_roi roi;
    int rc = roi_of(img, &roi);
    if (rc != HL_NO_ERROR)
        return rc;
    hl_geom g;
    if ((rc = hl_geometry(h, roi.w, roi.h, &g)) != HL_NO_ERROR)
        return rc;
    if ((rc = ensure_image(h, g, roi.w, roi.h)) != HL_NO_ERROR)
        return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int ntiles = g.tiles_x * g.tiles_y;
    hl_compact_args ca;
    memset(&ca, 0, sizeof(ca));
    ca.roi = roi;
    ca.tiles_x = g.tiles_x;
    ca.ntiles = ntiles;
    ca.imgs = nullptr;
    ca.group_img = nullptr;
    ca.nimg = 0;
    ca.ngroups = 0;
    ca.tile_state = h->d_tile_state;
    ca.ticket = reinterpret_cast<unsigned *>(h->d_counters + 3);
    ca.ticket_base = h->ticket_base;
    if (++h->epoch >= (1u << 30)) {
        CK(cudaMemsetAsync(h->d_tile_state, 0,
                           sizeof(unsigned long long) * h->cap_tiles, s));
        h->epoch = 1;
    }
    ca.epoch = h->epoch;
    ca.pts = pts_dev;
    ca.pts_f2 = nullptr;
    ca.tile_off = tile_off_dev;
    ca.count = count_dev;
    ca.status = h->d_counters + 1;
    {
        /* about one CTA per SM when they fit at once, else one per group */
        const int nct = hl_compact_persist_ctas(ntiles, h->sms);
        if (nct > 0) {
            CK(hl_launch_compact_persist(&ca, nct, s));
            h->ticket_base += (unsigned)nct;
        } else {
            CK(hl_launch_compact(&ca, s));
            h->ticket_base += (unsigned)((ntiles + HL_COMPACT_GROUP - 1) / HL_COMPACT_GROUP);
        }
    }
    h->last_launches = 1;
    return HL_NO_ERROR;
}

extern "C" int hl_accumulator(hl_handle *h, const hl_image_desc *img,
                              int32_t *acc_dev, void *stream)
{
    if (!h || !img || !acc_dev)
        return HL_NULL_POINTER;
    hl_roi roi;
    int rc = roi_of(img, &roi);
    if (rc != HL_NO_ERROR)
        return rc;
    hl_geom g;
    if ((rc = hl_geometry(h, roi.w, roi.h, &g)) != HL_NO_ERROR)
        return rc;
    if ((rc = ensure_image(h, g, roi.w, roi.h)) != HL_NO_ERROR)
        return rc;
    if ((rc = ensure_acc(h, g.numrho, 1)) != HL_NO_ERROR)
        return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int launches = 0;
    if ((rc = run_ab(h, roi, g, s, &launches)) != HL_NO_ERROR)
        return rc;
    CK(hl_launch_to_tight(h->d_acc, g.numrho, h->T, h->Tp, acc_dev, s));
    h->last_launches = launches + 1;
    return HL_NO_ERROR;
}

extern "C" int hl_accumulator_ref_layout(hl_handle *h, const hl_image_desc *img,
                                         int32_t *ref_dev, void *stream)
{
    if (!h || !img || !ref_dev)
        return HL_NULL_POINTER;
    hl_roi roi;
    int rc = roi_of(img, &roi);
    if (rc != HL_NO_ERROR)
        return rc;
    hl_geom g;
    if ((rc = hl_geometry(h, roi.w, roi.h, &g)) != HL_NO_ERROR)
        return rc;
    if ((rc = ensure_image(h, g, roi.w, roi.h)) != HL_NO_ERROR)
        return rc;
    if ((rc = ensure_acc(h, g.numrho, 1)) != HL_NO_ERROR)
        return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int launches = 0;
    if ((rc = run_ab(h, roi, g, s, &launches)) != HL_NO_ERROR)
        return rc;
    CK(hl_launch_to_ref(h->d_acc, g.numrho, h->T, h->Tp, g.rho_min,
                        g.ref_numrho, ref_dev, s));
    h->last_launches = launches + 1;
    return HL_NO_ERROR;
}

extern "C" int hl_lines_from_accumulator(hl_handle *h, const int32_t *acc_dev,
                                         int w, int hh, int *linesmax,
                                         hl_line *lines, void *stream)
{
    if (!h || !acc_dev || !linesmax)
        return HL_NULL_POINTER;
    if (*linesmax > 0 && !lines)
        return HL_NULL_POINTER;
    hl_geom g;
    int rc = hl_geometry(h, w, hh, &g);
    if (rc != HL_NO_ERROR)
        return rc;
    if ((rc = ensure_acc(h, g.numrho, *linesmax)) != HL_NO_ERROR)
        return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    CK(hl_launch_from_tight(acc_dev, g.numrho, h->T, h->Tp, h->d_acc, s));
    h->prof_open = 0;
    int launches = 1;
    if ((rc = run_c(h, g, *linesmax, nullptr, nullptr, s, &launches)) !=
        HL_NO_ERROR)
        return rc;
    h->last_launches = launches;
    return fetch_result(h, linesmax, lines, s);
}

extern "C" int hl_plain_points(hl_handle *h, const int *xy_dev, int n,
                               int *linesmax, hl_line *lines, void *stream)
{
    if (!h || !xy_dev || !linesmax)
        return HL_NULL_POINTER;
    if (*linesmax > 0 && !lines)
        return HL_NULL_POINTER;
    if (n <= 0)
        return HL_INVALID_DATA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int init[4] = {0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000};
    CK(cudaMemcpyAsync(h->d_counters + 4, init, sizeof(init),
                       cudaMemcpyHostToDevice, s));
    CK(hl_launch_bbox(xy_dev, n, h->d_counters + 4, s));
    int bb[4];
    CK(cudaMemcpyAsync(bb, h->d_counters + 4, sizeof(bb), cudaMemcpyDeviceToHost,
                       s));
    CK(cudaStreamSynchronize(s));
    /* the reference's accumulator height uses the box extent,
     * okano_3_0/HoughLine.cu:374-375,387 */
    int w = bb[2] - bb[0], hh = bb[3] - bb[1];
    double ax = std::max(fabs((double)bb[0]), fabs((double)bb[2]));
    double ay = std::max(fabs((double)bb[1]), fabs((double)bb[3]));
    hl_geom g;
    g.numtheta = h->T;
    g.theta_pad = h->Tp;
    layout(h, sqrt(ax * ax + ay * ay) + 1.0, &g.rho_min, &g.numrho);
    g.ref_numrho = (int)((double)(int)((w + hh) * 2 + 1) / h->p.derho);
    if ((double)g.numrho * h->Tp >= 2147483647.0)
        return HL_OP_OVERFLOW;
    int rc = ensure_acc(h, g.numrho, *linesmax);
    if (rc != HL_NO_ERROR)
        return rc;
    int rows, nwin, threads;
    vote_shape(h, g.numrho, &rows, &nwin, &threads);
    CK(hl_launch_vote_points(xy_dev, n, h->d_cos, h->d_sin, h->T, h->Tp,
                             g.rho_min, g.numrho, rows, nwin,
                             (float)(1.0 / h->p.derho), h->d_acc, threads, s));
    int launches = 2;
    h->prof_open = 0;
    if ((rc = run_c(h, g, *linesmax, nullptr, nullptr, s, &launches)) !=
        HL_NO_ERROR)
        return rc;
    h->last_launches = launches;
    return fetch_result(h, linesmax, lines, s);
}

extern "C" int hl_measure_smem_atomic_peak(int iters, double *atomics_per_s,
                                           void *stream)
{
    if (!atomics_per_s)
        return HL_NULL_POINTER;
    if (iters <= 0)
        return HL_INVALID_DATA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int *sink = nullptr;
    CK(cudaMalloc(&sink, sizeof(int)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int blocks = 0, threads = 0;
    cudaError_t e = hl_launch_atomic_bench(iters / 4 + 1, sink, s, &blocks,
                                           &threads);   /* warm-up */
    float best = 1e30f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; rep++) {
        cudaEventRecord(e0, s);
        e = hl_launch_atomic_bench(iters, sink, s, &blocks, &threads);
        cudaEventRecord(e1, s);
        if (e == cudaSuccess)
            e = cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess)
        return map_err(e);
    double total = (double)blocks * threads * (double)iters * 8.0;
    *atomics_per_s = total / (best * 1e-3);
    return HL_NO_ERROR;
}

extern "C" int hl_plain_draw(hl_handle *h, const hl_image_desc *in,
                             const hl_image_desc *out, int *linesmax,
                             hl_line *lines, void *stream)
{
    if (!h || !in || !out || !linesmax || !out->data)
        return HL_NULL_POINTER;
    if (*linesmax > 0 && !lines)
        return HL_NULL_POINTER;
    hl_roi rin, rout;
    int rc = roi_of(in, &rin);
    if (rc != HL_NO_ERROR)
        return rc;
    if ((rc = roi_of(out, &rout)) != HL_NO_ERROR)
        return rc;
    /* okano_3_0/HoughLine.cu:1101-1109: both ROIs shrink to the smaller
     * width and height; the accumulator height still comes from the input
     * ROI (:670), which only the decode sees */
    const int ref_nrho = (int)((double)(int)((rin.w + rin.h) * 2 + 1) / h->p.derho);
    const int w = std::min(rin.w, rout.w), hh = std::min(rin.h, rout.h);
    hl_image_desc vin = *in;
    vin.roi_x2 = vin.roi_x1 + w;
    vin.roi_y2 = vin.roi_y1 + hh;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    rc = plain_launch(h, &vin, *linesmax, nullptr, nullptr, s, ref_nrho);
    if (rc != HL_NO_ERROR)
        return rc;
    const int launches = h->last_launches;
    rc = fetch_result(h, linesmax, lines, s);
    if (rc != HL_NO_ERROR)
        return rc;
    if (*linesmax > 0) {
        /* the drawing kernel reads the records still held in the device
         * result block */
        const hl_line *dl = reinterpret_cast<const hl_line *>(h->d_result +
                                                              sizeof(hl_result_hdr));
        int derho_i = (int)h->p.derho;   /* _houghoutKer takes an int derho */
        if (derho_i == 0)
            return HL_INVALID_DATA;
        CK(hl_launch_draw(const_cast<uint8_t *>(rout.base), rout.pitch, w, hh, dl,
                          *linesmax, derho_i, s));
        CK(cudaStreamSynchronize(s));
        h->last_launches = launches + (*linesmax + 1023) / 1024;
    }
    return HL_NO_ERROR;
}

extern "C" int hl_draw_lines(hl_handle *h, const hl_image_desc *out,
                             const hl_line *lines, int nlines, void *stream)
{
    if (!h || !out)
        return HL_NULL_POINTER;
    if (nlines <= 0)
        return HL_NO_ERROR;
    if (!lines)
        return HL_NULL_POINTER;
    hl_roi r;
    int rc = roi_of(out, &r);
    if (rc != HL_NO_ERROR)
        return rc;
    int derho_i = (int)h->p.derho;
    if (derho_i == 0)
        return HL_INVALID_DATA;
    size_t bytes = sizeof(hl_result_hdr) + sizeof(hl_line) * (size_t)nlines;
    if ((rc = grow((void **)&h->d_aux, &h->cap_aux, bytes)) != HL_NO_ERROR)
        return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaMemcpyAsync(h->d_aux, lines, sizeof(hl_line) * (size_t)nlines,
                       cudaMemcpyHostToDevice, s));
    CK(hl_launch_draw(const_cast<uint8_t *>(r.base), r.pitch, r.w, r.h,
                      reinterpret_cast<const hl_line *>(h->d_aux), nlines,
                      derho_i, s));
    CK(cudaStreamSynchronize(s));
    h->last_launches = (nlines + 1023) / 1024;
    return HL_NO_ERROR;
}

extern "C" int hl_real_line(hl_handle *h, const hl_image_desc *img, int x1,
                            int y1, int x2, int y2, float threshold,
                            float thresperc, int *is_real, int *pointnum,
                            void *stream)
{
    if (!h || !img || !is_real)
        return HL_NULL_POINTER;
    hl_roi roi;
    int rc = roi_of(img, &roi);
    if (rc != HL_NO_ERROR)
        return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int *cnt = h->d_counters + 8;
    CK(cudaMemsetAsync(cnt, 0, sizeof(int), s));
    /* okano_3_0/HoughLine.cu:1436-1443: the float threshold is passed to an
     * int parameter (truncation) */
    CK(hl_launch_real_line(roi.base, roi.pitch, roi.w, roi.h, x1, y1, x2, y2,
                           (int)threshold, cnt, s));
    int n = 0;
    CK(cudaMemcpyAsync(&n, cnt, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    /* :1405: int pointnumfull = sqrt(0.0 + dx*dx + dy*dy) */
    const int full = (int)sqrt(0.0 + (double)(x1 - x2) * (x1 - x2) +
                               (double)(y1 - y2) * (y1 - y2));
    *is_real = ((float)n > (float)full * thresperc) ? 1 : 0;
    if (pointnum)
        *pointnum = n;
    h->last_launches = 1;
    return HL_NO_ERROR;
}

/* ==================================================================== */
/* Batched path                                                          */
/* ==================================================================== */

/* Counters of a batch call, cleared at its start: [0] compaction ticket,
 * [1] vote work counter, [2] status word, [3] total points, [8] noted peak
 * candidates. */
#define BW_NCNT 16

struct hl_batch_ws {
    float2 *d_pts;
    size_t cap_pts;
    unsigned long long *d_state;   /* look-back state per 4-tile group */
    size_t cap_state;
    int *d_tile_off;
    size_t cap_tile_off;
    int32_t *d_acc;
    size_t cap_acc;
    unsigned long long *d_keys;
    size_t cap_keys;
    unsigned long long *d_cand;    /* noted peak candidates; counter d_cnt[8] */
    size_t cap_cand;
    int4 *d_scratch;               /* split parts' slots: win_rows x HL_SLICE */
    size_t cap_scratch;
    unsigned *d_tmask;             /* every image's admitted-tile masks */
    size_t cap_tmask;
    int masks_dirty;               /* the plan changed: recompute them */
    int *d_ncand;                  /* per image, zero between calls */
    size_t cap_ncand;
    int *d_cnt;
    unsigned char *d_tab;          /* per-image tables of one call */
    size_t cap_tab;
    unsigned char *h_tab;          /* their pinned staging copy */
    size_t cap_htab;
    hl_line *d_lines;              /* hl_batch's device results */
    size_t cap_lines;
    int *d_counts;
    size_t cap_counts;
    unsigned char *h_res;          /* pinned copy of results + status */
    size_t cap_hres;
    cudaEvent_t tab_read;          /* the previous call's table upload */
    int tab_event;

    /* the plan of the last call (reused while the geometry is the same) */
    std::vector<int> key;
    size_t tab_bytes;
    size_t off_cimg, off_gimg, off_vimg, off_items, off_pimg, off_chunks,
        off_fimg, off_merge;
    int ngroups, ntiles, nitems, nchunks, grid, threads, win_rows;
    size_t npts_cap, acc_ints, nkeys;
    std::vector<size_t> acc_off, key_off;
    std::vector<size_t> pts_base;  /* each image's first point */
    std::vector<int> key_cap_i, tile_base, group_base, nwin, rho_min, R,
        ref_numrho;
    std::vector<int4> items;
    std::vector<hl_merge_region> merge; /* the split blocks */
    int nslots;                    /* scratch slots of their parts */
    int part16;                    /* 16-bit slots (hl_part16_ok for all) */
    std::vector<size_t> tmask_off; /* each image's first mask word */
    size_t tmask_words, max_mask_words;
    std::vector<int2> chunks;
    std::vector<int> group_img;

    /* captured pipeline (captured on a private stream: the caller's may be
     * the legacy default stream, which cannot be captured) */
    cudaStream_t cap_stream;
    cudaGraphExec_t gexec;
    std::vector<long long> gkey;
};

static void batch_ws_free(hl_batch_ws *b);
static void prop_free(hl_handle *h);

static void batch_free(hl_handle *h)
{
    batch_ws_free(h->bw);
    batch_ws_free(h->bw_fb);
    h->bw = h->bw_fb = nullptr;
    prop_free(h);
}

static void batch_ws_free(hl_batch_ws *b)
{
    if (!b)
        return;
    void *dp[] = {b->d_pts, b->d_state, b->d_tile_off, b->d_acc, b->d_keys, b->d_cand,
                  b->d_ncand, b->d_cnt, b->d_tab, b->d_lines, b->d_counts,
                  b->d_scratch, b->d_tmask};
    for (void *q : dp)
        if (q)
            cudaFree(q);
    if (b->h_tab)
        cudaFreeHost(b->h_tab);
    if (b->h_res)
        cudaFreeHost(b->h_res);
    if (b->tab_event)
        cudaEventDestroy(b->tab_read);
    if (b->gexec)
        cudaGraphExecDestroy(b->gexec);
    if (b->cap_stream)
        cudaStreamDestroy(b->cap_stream);
    delete b;
}

static int grow_host(unsigned char **ptr, size_t *cap, size_t need)
{
    if (*cap >= need && *ptr)
        return HL_NO_ERROR;
    size_t nb = std::max(need, (size_t)4096);
    nb += nb / 4;
    if (*ptr)
        cudaFreeHost(*ptr);
    *ptr = nullptr;
    *cap = 0;
    CK(cudaMallocHost(ptr, nb));
    *cap = nb;
    return HL_NO_ERROR;
}

static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

/* Per-image rho-window weights of the vote items on an 8 x 8 grid of cell
 * centres (the image's share of points in each (slice, window) block when
 * edges are spread evenly), in units of pixels. */
static void batch_block_weights(const hl_handle *h, int w, int hh, int rho_min,
                                int rows, int nwin, std::vector<double> &wt)
{
    const int slices = h->Tp / HL_SLICE;
    wt.assign((size_t)slices * nwin, 0.0);
    const int G = 8;
    const double cell = (double)w * hh / (G * G);
    for (int sl = 0; sl < slices; sl++) {
        const int k0 = sl * HL_SLICE;
        const int k1 = std::min(k0 + HL_SLICE, h->T) - 1;
        if (k0 >= h->T)
            continue;
        const double th = 0.5 * (k0 + k1) * h->p.detheta;
        const double c = cos(th), sn = sin(th);
        for (int gy = 0; gy < G; gy++) {
            const double y = (gy + 0.5) * hh / G;
            for (int gx = 0; gx < G; gx++) {
                const double x = (gx + 0.5) * w / G;
                const int row = (int)floor((x * c + y * sn) / h->p.derho) - rho_min;
                const int wn = std::min(std::max(row / rows, 0), nwin - 1);
                wt[(size_t)sl + (size_t)slices * wn] += cell;   /* 32 lanes per point */
            }
        }
    }
}

/* Plan a batch: sizes, offsets, work items, chunks; fills the pinned tables
 * (image pointers and thresholds included).  The geometry part is reused
 * when the sizes and the launch shape equal the previous call's. */
static int batch_plan(hl_handle *h, hl_batch_ws *b, const hl_image_desc *imgs,
                      int nimg, const int *thr, int K, hl_line *lines_dev,
                      int *counts_dev, const hl_roi *rois)
{
    const int slices = h->Tp / HL_SLICE;
    int maxR = 1;
    std::vector<hl_geom> gs((size_t)nimg);
    for (int i = 0; i < nimg; i++) {
        int rc = hl_geometry(h, rois[i].w, rois[i].h, &gs[i]);
        if (rc != HL_NO_ERROR)
            return rc;
        maxR = std::max(maxR, gs[i].numrho);
    }
    /* launch shape: the override (autotuner) or the largest window that
     * fits, 1024 threads */
    const int maxr = hl_vote_max_rows();
    int rows = h->win_rows_override > 0 ? std::min(h->win_rows_override, maxr)
                                        : std::min(maxR, maxr);
    rows = std::max(8, (rows + 7) / 8 * 8);
    rows = std::min(rows, maxr);
    const int threads = h->threads_override > 0 ? h->threads_override : 1024;
    const size_t smem = hl_vote_smem_bytes(rows);
    const int per_sm = std::max(1, std::min(2048 / threads,
                                            (int)((228u * 1024u) / (smem + 1024))));
    const int ctas = std::max(h->sms, 1) * per_sm;

    std::vector<int> key;
    key.reserve(2 * (size_t)nimg + 8);
    key.push_back(nimg);
    key.push_back(rows);
    key.push_back(threads);
    key.push_back(h->T);
    {   /* derho sets every image's rho range */
        unsigned long long bits;
        memcpy(&bits, &h->p.derho, sizeof(bits));
        key.push_back((int)(bits & 0xffffffffu));
        key.push_back((int)(bits >> 32));
    }
    for (int i = 0; i < nimg; i++) {
        key.push_back(rois[i].w);
        key.push_back(rois[i].h);
    }
    if (key != b->key) {
        b->key = key;
        b->win_rows = rows;
        b->threads = threads;
        b->acc_off.assign(nimg, 0);
        b->key_off.assign(nimg, 0);
        b->key_cap_i.assign(nimg, 0);
        b->tile_base.assign(nimg, 0);
        b->group_base.assign(nimg, 0);
        b->nwin.assign(nimg, 0);
        b->rho_min.assign(nimg, 0);
        b->R.assign(nimg, 0);
        b->ref_numrho.assign(nimg, 0);
        b->group_img.clear();
        b->chunks.clear();
        size_t acc = 0, keys = 0, pts = 0;
        b->pts_base.assign(nimg, 0);
        int tiles = 0, groups = 0;
        b->tmask_off.assign(nimg, 0);
        b->tmask_words = 0;
        b->max_mask_words = 0;
        b->masks_dirty = 1;
        std::vector<double> allw;
        std::vector<int2> blocks;
        std::vector<double> wt;
        for (int i = 0; i < nimg; i++) {
            const hl_geom &g = gs[i];
            const int nt = g.tiles_x * g.tiles_y;
            const int ng = (nt + HL_COMPACT_GROUP - 1) / HL_COMPACT_GROUP;
            b->tile_base[i] = tiles;
            b->group_base[i] = groups;
            for (int q = 0; q < ng; q++)
                b->group_img.push_back(i);
            tiles += nt + 1;   /* the image's tile offsets and its end */
            groups += ng;
            /* room for every pixel and one pad per tile, kept even so every
             * image's point list starts on 16 bytes */
            b->pts_base[i] = pts;
            pts += ((size_t)rois[i].w * rois[i].h + (size_t)nt + 16 + 1) & ~(size_t)1;
            b->acc_off[i] = acc;
            acc += (size_t)g.numrho * h->Tp;
            /* peak-key capacity: the bound of ensure_acc, at most 2^17 */
            const size_t kc = std::min((size_t)g.numrho * ((h->T + 1) / 2) + 32,
                                       (size_t)1 << 17);
            b->key_off[i] = keys;
            b->key_cap_i[i] = (int)kc;
            keys += kc;
            b->rho_min[i] = g.rho_min;
            b->R[i] = g.numrho;
            b->ref_numrho[i] = g.ref_numrho;
            b->nwin[i] = (g.numrho + rows - 1) / rows;
            {
                const size_t mw = hl_tile_mask_words(slices, b->nwin[i], nt);
                b->tmask_off[i] = b->tmask_words;
                b->tmask_words += mw;
                b->max_mask_words = std::max(b->max_mask_words, mw);
            }
            for (int r0 = 0; r0 < g.numrho; r0 += HL_PEAK_ROWS)
                b->chunks.push_back(make_int2(i, r0));
            if ((size_t)slices * b->nwin[i] > 0xffff)
                return HL_OP_OVERFLOW;   /* ... and the block in 16 bits */
            batch_block_weights(h, rois[i].w, rois[i].h, g.rho_min, rows,
                                b->nwin[i], wt);
            for (size_t q = 0; q < wt.size(); q++) {
                blocks.push_back(make_int2(i, (int)q));
                allw.push_back(wt[q]);
            }
        }
        if (nimg > 0xffff)
            return HL_OP_OVERFLOW;   /* the item packs the image in 16 bits */
        /* items: plan_parts over every image's blocks (a block heavier
         * than a third of one CTA's share is split); the parts of a split
         * block vote into scratch slots, summed into it by the merge
         * launch */
        std::vector<int> pieces;
        const std::vector<vote_part> parts = plan_parts(allw, ctas, 3.0, pieces);
        b->merge.clear();
        std::vector<int> slot0(blocks.size(), 0), used(blocks.size(), 0);
        int nslots = 0;
        for (size_t q = 0; q < blocks.size(); q++) {
            if (pieces[q] <= 1)
                continue;
            const int im = blocks[q].x, blk = blocks[q].y;
            const int w0 = (blk / slices) * rows, k0 = (blk % slices) * HL_SLICE;
            const long long off = (long long)b->acc_off[im] + (long long)w0 * h->Tp + k0;
            slot0[q] = nslots;
            b->merge.push_back({off / 4, std::min(rows, b->R[im] - w0), k0, nslots, pieces[q],
                                w0, im, {0, 0}});
            nslots += pieces[q];
        }
        b->items.resize(parts.size());
        for (size_t q = 0; q < parts.size(); q++) {
            const vote_part &p = parts[q];
            const int slot = pieces[p.blk] > 1 ? slot0[p.blk] + used[p.blk]++ : 0;
            b->items[q] = make_int4(blocks[p.blk].y | (blocks[p.blk].x << 16),
                                    p.part | (p.nparts << 16), slot, 0);
        }
        b->nslots = nslots;
        b->part16 = 1;
        for (int i = 0; i < nimg; i++)
            b->part16 &= hl_part16_ok(h->p.derho, rois[i].w, rois[i].h);
        b->ngroups = groups;
        b->ntiles = tiles;
        b->nitems = (int)b->items.size();
        b->nchunks = (int)b->chunks.size();
        b->grid = std::max(1, std::min(b->nitems, ctas));
        b->npts_cap = pts;
        b->acc_ints = acc;
        b->nkeys = keys;
        /* table layout */
        size_t o = 0;
        b->off_cimg = o;   o = align16(o + sizeof(hl_compact_img) * nimg);
        b->off_gimg = o;   o = align16(o + sizeof(int) * (size_t)groups);
        b->off_vimg = o;   o = align16(o + sizeof(hl_vote_img) * nimg);
        b->off_items = o;  o = align16(o + sizeof(int4) * b->items.size());
        b->off_merge = o;  o = align16(o + sizeof(hl_merge_region) * b->merge.size());
        b->off_pimg = o;   o = align16(o + sizeof(hl_peak_img) * nimg);
        b->off_chunks = o; o = align16(o + sizeof(int2) * b->chunks.size());
        b->off_fimg = o;   o = align16(o + sizeof(hl_final_img) * nimg);
        b->tab_bytes = o;
    }

    /* device buffers */
    int rc;
    if ((rc = grow((void **)&b->d_pts, &b->cap_pts, sizeof(float2) * b->npts_cap)) != HL_NO_ERROR ||
        (rc = grow((void **)&b->d_state, &b->cap_state,
                   sizeof(unsigned long long) * ((size_t)b->ngroups + 1))) != HL_NO_ERROR ||
        (rc = grow((void **)&b->d_tile_off, &b->cap_tile_off,
                   sizeof(int) * ((size_t)b->ntiles + 1))) != HL_NO_ERROR ||
        (rc = grow((void **)&b->d_acc, &b->cap_acc, sizeof(int32_t) * b->acc_ints)) != HL_NO_ERROR ||
        (rc = grow((void **)&b->d_cand, &b->cap_cand,
                   sizeof(unsigned long long) * (65536 + b->acc_ints / 128))) != HL_NO_ERROR ||
        (rc = grow((void **)&b->d_keys, &b->cap_keys,
                   sizeof(unsigned long long) * b->nkeys)) != HL_NO_ERROR ||
        (rc = grow((void **)&b->d_tab, &b->cap_tab, b->tab_bytes)) != HL_NO_ERROR ||
        (rc = grow((void **)&b->d_scratch, &b->cap_scratch,
                   sizeof(int4) * (size_t)std::max(b->nslots, 1) * b->win_rows *
                       (HL_SLICE / 4))) != HL_NO_ERROR ||
        (rc = grow_tracked((void **)&b->d_tmask, &b->cap_tmask,
                           sizeof(unsigned) * std::max(b->tmask_words, (size_t)1),
                           &b->masks_dirty)) != HL_NO_ERROR)
        return rc;
    if (b->cap_ncand < sizeof(int) * (size_t)nimg || !b->d_ncand) {
        if ((rc = grow((void **)&b->d_ncand, &b->cap_ncand, sizeof(int) * (size_t)nimg)) !=
            HL_NO_ERROR)
            return rc;
        CK(cudaMemset(b->d_ncand, 0, b->cap_ncand));
    }
    if (!b->d_cnt)
        CK(cudaMalloc(&b->d_cnt, BW_NCNT * sizeof(int)));
    /* the previous call's upload must be done before the staging is reused */
    if (b->tab_event)
        CK(cudaEventSynchronize(b->tab_read));
    if ((rc = grow_host(&b->h_tab, &b->cap_htab, b->tab_bytes)) != HL_NO_ERROR)
        return rc;

    /* tables */
    unsigned char *t = b->h_tab;
    hl_compact_img *ci = reinterpret_cast<hl_compact_img *>(t + b->off_cimg);
    hl_vote_img *vi = reinterpret_cast<hl_vote_img *>(t + b->off_vimg);
    hl_peak_img *pi = reinterpret_cast<hl_peak_img *>(t + b->off_pimg);
    hl_final_img *fi = reinterpret_cast<hl_final_img *>(t + b->off_fimg);
    for (int i = 0; i < nimg; i++) {
        const hl_geom &g = gs[i];
        const int nt = g.tiles_x * g.tiles_y;
        ci[i].roi = rois[i];
        ci[i].tiles_x = g.tiles_x;
        ci[i].ntiles = nt;
        ci[i].tile_base = b->tile_base[i];
        ci[i].group_base = b->group_base[i];
        ci[i].ngroups = (nt + HL_COMPACT_GROUP - 1) / HL_COMPACT_GROUP;
        ci[i].pad = 0;
        ci[i].pts_base = (long long)b->pts_base[i];
        vi[i].pts = b->d_pts + b->pts_base[i];
        vi[i].tile_off = b->d_tile_off + b->tile_base[i];
        vi[i].ntiles = nt;
        vi[i].tiles_x = g.tiles_x;
        vi[i].w = rois[i].w;
        vi[i].h = rois[i].h;
        vi[i].rho_min = g.rho_min;
        vi[i].R = g.numrho;
        vi[i].nwin = b->nwin[i];
        vi[i].threshold = thr ? thr[i] : h->p.threshold;
        vi[i].tmask = b->d_tmask + b->tmask_off[i];
        vi[i].acc = b->d_acc + b->acc_off[i];
        pi[i].acc = b->d_acc + b->acc_off[i];
        pi[i].keys = b->d_keys + b->key_off[i];
        pi[i].ncand = b->d_ncand + i;
        pi[i].R = g.numrho;
        pi[i].cap = b->key_cap_i[i];
        pi[i].threshold = thr ? thr[i] : h->p.threshold;
        pi[i].pad = 0;
        fi[i].keys = b->d_keys + b->key_off[i];
        fi[i].ncand = b->d_ncand + i;
        fi[i].cap = b->key_cap_i[i];
        fi[i].rho_min = g.rho_min;
        fi[i].ref_numrho = g.ref_numrho;
        fi[i].pad = 0;
        fi[i].lines = lines_dev + (size_t)i * (size_t)std::max(K, 0);
        fi[i].count_out = counts_dev + i;
    }
    memcpy(t + b->off_gimg, b->group_img.data(), sizeof(int) * b->group_img.size());
    memcpy(t + b->off_items, b->items.data(), sizeof(int4) * b->items.size());
    if (!b->merge.empty())
        memcpy(t + b->off_merge, b->merge.data(), sizeof(hl_merge_region) * b->merge.size());
    memcpy(t + b->off_chunks, b->chunks.data(), sizeof(int2) * b->chunks.size());
    return HL_NO_ERROR;
}

/* The stream work of one planned batch call. */
/* counters, look-back states, tables, then the compaction of every image */
static int batch_enqueue_compact(hl_handle *h, hl_batch_ws *b, int nimg,
                                 cudaStream_t s)
{
    unsigned char *dt = b->d_tab;
    CK(cudaMemsetAsync(b->d_cnt, 0, BW_NCNT * sizeof(int), s));
    CK(cudaMemsetAsync(b->d_state, 0,
                       sizeof(unsigned long long) * ((size_t)b->ngroups + 1), s));
    CK(cudaMemcpyAsync(dt, b->h_tab, b->tab_bytes, cudaMemcpyHostToDevice, s));

    hl_compact_args ca;
    memset(&ca, 0, sizeof(ca));
    ca.imgs = reinterpret_cast<const hl_compact_img *>(dt + b->off_cimg);
    ca.group_img = reinterpret_cast<const int *>(dt + b->off_gimg);
    ca.nimg = nimg;
    ca.ngroups = b->ngroups;
    ca.tile_state = b->d_state;
    ca.ticket = reinterpret_cast<unsigned *>(b->d_cnt + 0);
    ca.ticket_base = 0;
    ca.epoch = 1;
    ca.pts = nullptr;
    ca.pts_f2 = b->d_pts;
    ca.tile_off = b->d_tile_off;
    ca.count = b->d_cnt + 3;
    ca.status = b->d_cnt + 2;
    CK(hl_launch_compact(&ca, s));
    prof_mark(h, 1, s);
    return HL_NO_ERROR;
}

/* the full vote and the peak pass */
static int batch_enqueue_vote_peaks(hl_handle *h, hl_batch_ws *b, cudaStream_t s)
{
    unsigned char *dt = b->d_tab;
    hl_vote_args va;
    memset(&va, 0, sizeof(va));
    va.imgs = reinterpret_cast<const hl_vote_img *>(dt + b->off_vimg);
    va.cosv = h->d_cos;
    va.sinv = h->d_sin;
    va.T = h->T;
    va.Tp = h->Tp;
    va.win_rows = b->win_rows;
    va.irho = (float)(1.0 / h->p.derho);   /* okano_3_0/HoughLine.cu:107 */
    va.status = b->d_cnt + 2;
    va.items = reinterpret_cast<const int4 *>(dt + b->off_items);
    va.nitems = b->nitems;
    va.scratch = b->d_scratch;
    va.part16 = b->part16;
    /* the counter is cleared with the others at the start of every call */
    va.cand = cand_list(b->d_cand, b->cap_cand, b->d_cnt + 8);
    va.work = reinterpret_cast<unsigned *>(b->d_cnt + 1);
    va.work_base = 0;
    CK(hl_launch_vote(&va, b->threads, b->grid, s));
    if (!b->merge.empty()) {
        hl_merge_args ma;
        ma.acc = reinterpret_cast<int4 *>(b->d_acc);
        ma.pitch4 = h->Tp / 4;
        ma.T = h->T;
        ma.scratch = b->d_scratch;
        ma.slot4 = hl_slot4(b->win_rows, b->part16);
        ma.regs = reinterpret_cast<const hl_merge_region *>(dt + b->off_merge);
        ma.nreg = (int)b->merge.size();
        ma.part16 = b->part16;
        ma.pimgs = reinterpret_cast<const hl_peak_img *>(dt + b->off_pimg);
        ma.thr0 = 0;
        ma.cand = va.cand;
        CK(hl_launch_merge(&ma, b->win_rows, s));
    }
    prof_mark(h, 2, s);

    hl_peak_args pa;
    memset(&pa, 0, sizeof(pa));
    pa.imgs = reinterpret_cast<const hl_peak_img *>(dt + b->off_pimg);
    pa.chunks = reinterpret_cast<const int2 *>(dt + b->off_chunks);
    pa.nchunks = b->nchunks;
    pa.T = h->T;
    pa.Tp = h->Tp;
    pa.status = b->d_cnt + 2;
    pa.cand = va.cand;
    CK(hl_launch_peaks(&pa, s));
    prof_mark(h, 3, s);
    return HL_NO_ERROR;
}

/* rank, merge and write the lines of every image */
static int batch_enqueue_finalize(hl_handle *h, hl_batch_ws *b, int nimg, int K,
                                  cudaStream_t s)
{
    unsigned char *dt = b->d_tab;
    hl_final_args fa;
    memset(&fa, 0, sizeof(fa));
    fa.imgs = reinterpret_cast<const hl_final_img *>(dt + b->off_fimg);
    fa.T = h->T;
    fa.detheta = h->p.detheta;
    fa.thresdis = h->p.thresdis;
    fa.thresang = h->p.thresang;
    fa.linesmax = K;
    fa.hdr = nullptr;
    fa.status = b->d_cnt + 2;
    CK(hl_launch_finalize(&fa, nimg, s));
    prof_mark(h, 4, s);
    return HL_NO_ERROR;
}

static int batch_enqueue(hl_handle *h, hl_batch_ws *b, int nimg, int K,
                         cudaStream_t s)
{
    int rc;
    if ((rc = batch_enqueue_compact(h, b, nimg, s)) != HL_NO_ERROR ||
        (rc = batch_enqueue_vote_peaks(h, b, s)) != HL_NO_ERROR)
        return rc;
    return batch_enqueue_finalize(h, b, nimg, K, s);
}

static int batch_run_ws(hl_handle *h, hl_batch_ws **pb, const hl_image_desc *imgs,
                        int nimg, const int *thr, int K, hl_line *lines_dev,
                        int *counts_dev, cudaStream_t s)
{
    if (nimg <= 0)
        return HL_INVALID_DATA;
    if (!*pb) {
        *pb = new (std::nothrow) hl_batch_ws();
        if (!*pb)
            return HL_OUT_OF_MEM;
    }
    hl_batch_ws *b = *pb;
    std::vector<hl_roi> rois((size_t)nimg);
    for (int i = 0; i < nimg; i++) {
        int rc = roi_of(&imgs[i], &rois[i]);
        if (rc != HL_NO_ERROR)
            return rc;
    }
    int rc = batch_plan(h, b, imgs, nimg, thr, K, lines_dev, counts_dev, rois.data());
    if (rc != HL_NO_ERROR)
        return rc;
    h->last_batch = 1;
    h->last_launches = 4;
    if (!b->tab_event) {
        CK(cudaEventCreateWithFlags(&b->tab_read, cudaEventDisableTiming));
        b->tab_event = 1;
    }
    if (b->masks_dirty) {
        /* tile masks of the new plan, outside the (captured) pipeline: the
         * image table they read is the one the pipeline uploads again */
        CK(cudaMemcpyAsync(b->d_tab + b->off_vimg, b->h_tab + b->off_vimg,
                           sizeof(hl_vote_img) * (size_t)nimg, cudaMemcpyHostToDevice, s));
        hl_vote_args va;
        memset(&va, 0, sizeof(va));
        va.imgs = reinterpret_cast<const hl_vote_img *>(b->d_tab + b->off_vimg);
        va.cosv = h->d_cos;
        va.sinv = h->d_sin;
        va.T = h->T;
        va.Tp = h->Tp;
        va.win_rows = b->win_rows;
        va.irho = (float)(1.0 / h->p.derho);
        CK(hl_launch_tile_masks(&va, nimg, b->max_mask_words, s));
        b->masks_dirty = 0;
    }
    prof_mark(h, 0, s);
    if (!h->batch_graph || h->prof) {
        rc = batch_enqueue(h, b, nimg, K, s);
    } else {
        /* graph key: the plan key plus what the captured nodes hold */
        std::vector<long long> gk(b->key.begin(), b->key.end());
        gk.push_back((long long)(uintptr_t)lines_dev);
        gk.push_back((long long)(uintptr_t)counts_dev);
        gk.push_back(K);
        gk.push_back((long long)(uintptr_t)b->d_acc);
        gk.push_back((long long)(uintptr_t)b->d_pts);
        gk.push_back((long long)(uintptr_t)b->d_tab);
        gk.push_back((long long)(uintptr_t)b->h_tab);
        gk.push_back((long long)(uintptr_t)b->d_keys);
        gk.push_back((long long)(uintptr_t)b->d_tmask);
        gk.push_back((long long)(uintptr_t)b->d_scratch);
        gk.push_back((long long)(uintptr_t)b->d_cand);
        if (!b->gexec || gk != b->gkey) {
            if (b->gexec) {
                cudaGraphExecDestroy(b->gexec);
                b->gexec = nullptr;
            }
            if (!b->cap_stream)
                CK(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
            cudaGraph_t graph = nullptr;
            CK(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
            rc = batch_enqueue(h, b, nimg, K, b->cap_stream);
            cudaError_t e = cudaStreamEndCapture(b->cap_stream, &graph);
            if (rc != HL_NO_ERROR) {
                if (graph)
                    cudaGraphDestroy(graph);
                return rc;
            }
            if (e != cudaSuccess)
                return map_err(e);
            e = cudaGraphInstantiate(&b->gexec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                b->gexec = nullptr;
                return map_err(e);
            }
            b->gkey = gk;
        }
        CK(cudaGraphLaunch(b->gexec, s));
        h->last_launches = 4;
    }
    if (rc == HL_NO_ERROR)
        CK(cudaEventRecord(b->tab_read, s));
    return rc;
}

static int batch_run(hl_handle *h, const hl_image_desc *imgs, int nimg,
                     const int *thr, int K, hl_line *lines_dev,
                     int *counts_dev, cudaStream_t s)
{
    return batch_run_ws(h, &h->bw, imgs, nimg, thr, K, lines_dev, counts_dev, s);
}

static int batch_last_status(hl_handle *h, int *status, cudaStream_t s)
{
    hl_batch_ws *b = h->bw;
    if (!b || !b->d_cnt) {
        *status = 0;
        return HL_NO_ERROR;
    }
    int st = 0;
    CK(cudaMemcpyAsync(&st, b->d_cnt + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *status = st;
    return HL_NO_ERROR;
}

extern "C" int hl_set_batch_graph(hl_handle *h, int enable)
{
    if (!h)
        return HL_NULL_POINTER;
    h->batch_graph = enable ? 1 : 0;
    return HL_NO_ERROR;
}

extern "C" int hl_batch_async(hl_handle *h, const hl_image_desc *imgs, int nimg,
                              const int *thresholds, int linesmax,
                              hl_line *lines_dev, int *counts_dev, void *stream)
{
    if (!h || !imgs || !counts_dev)
        return HL_NULL_POINTER;
    if (linesmax > 0 && !lines_dev)
        return HL_NULL_POINTER;
    return batch_run(h, imgs, nimg, thresholds, linesmax, lines_dev, counts_dev,
                     reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int hl_tiles(hl_handle *h, const hl_image_desc *img, int piecenum, int linesmax,
                        hl_line *lines, int *counts, void *stream)
{
    if (!h || !img || !counts)
        return HL_NULL_POINTER;
    if (piecenum <= 0 || piecenum > 1024)
        return HL_INVALID_DATA;
    const int cx = img->width / piecenum, cy = img->height / piecenum;
    if (cx < 2 || cy < 2)
        return HL_INVALID_DATA;
    std::vector<hl_image_desc> cells((size_t)piecenum * piecenum, *img);
    for (int y = 0; y < piecenum; y++)
        for (int x = 0; x < piecenum; x++) {
            hl_image_desc &d = cells[(size_t)y * piecenum + x];
            d.roi_x1 = x * cx;
            d.roi_x2 = x * cx + cx - 1;   /* okano_3_0/HoughRec.cu:745-748 */
            d.roi_y1 = y * cy;
            d.roi_y2 = y * cy + cy - 1;
        }
    return hl_batch(h, cells.data(), (int)cells.size(), nullptr, linesmax, lines, counts,
                    stream);
}

extern "C" int hl_batch(hl_handle *h, const hl_image_desc *imgs, int nimg,
                        const int *thresholds, int linesmax, hl_line *lines,
                        int *counts, void *stream)
{
    if (!h || !imgs || !counts)
        return HL_NULL_POINTER;
    if (linesmax > 0 && !lines)
        return HL_NULL_POINTER;
    if (nimg <= 0)
        return HL_INVALID_DATA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (!h->bw) {
        h->bw = new (std::nothrow) hl_batch_ws();
        if (!h->bw)
            return HL_OUT_OF_MEM;
    }
    hl_batch_ws *b = h->bw;
    const size_t K = (size_t)std::max(linesmax, 0);
    int rc;
    if ((rc = grow((void **)&b->d_lines, &b->cap_lines,
                   sizeof(hl_line) * std::max(K * nimg, (size_t)1))) != HL_NO_ERROR ||
        (rc = grow((void **)&b->d_counts, &b->cap_counts, sizeof(int) * nimg)) != HL_NO_ERROR)
        return rc;
    rc = batch_run(h, imgs, nimg, thresholds, linesmax, b->d_lines, b->d_counts, s);
    if (rc != HL_NO_ERROR)
        return rc;
    const size_t lbytes = sizeof(hl_line) * K * nimg;
    if ((rc = grow_host(&b->h_res, &b->cap_hres, lbytes + sizeof(int) * (nimg + 1))) !=
        HL_NO_ERROR)
        return rc;
    int *h_counts = reinterpret_cast<int *>(b->h_res + lbytes);
    CK(cudaMemcpyAsync(h_counts, b->d_counts, sizeof(int) * nimg,
                       cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h_counts + nimg, b->d_cnt + 2, sizeof(int),
                       cudaMemcpyDeviceToHost, s));
    if (lbytes)
        CK(cudaMemcpyAsync(b->h_res, b->d_lines, lbytes, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (h_counts[nimg] != 0)
        return HL_CUDA_ERROR;
    for (int i = 0; i < nimg; i++) {
        const int c = std::max(0, std::min(h_counts[i], linesmax));
        counts[i] = c;
        if (c > 0)
            memcpy(lines + (size_t)i * K, b->h_res + sizeof(hl_line) * K * i,
                   sizeof(hl_line) * c);
    }
    return HL_NO_ERROR;
}

extern "C" int hl_autotune(hl_handle *h, const hl_image_desc *imgs, int nimg,
                           const int *thresholds, int linesmax,
                           hl_tune_entry *best, hl_tune_entry *tried,
                           int max_tried, int *ntried, void *stream)
{
    if (!h || !imgs || !best)
        return HL_NULL_POINTER;
    if (nimg <= 0)
        return HL_INVALID_DATA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int maxr = hl_vote_max_rows();
    const int row_cand[] = {256, 512, 768, 1024, maxr};
    const int thr_cand[] = {512, 1024};
    const int K = std::max(linesmax, 1);
    hl_line *d_lines = nullptr;
    int *d_counts = nullptr;
    CK(cudaMalloc(&d_lines, sizeof(hl_line) * (size_t)K * nimg));
    if (cudaMalloc(&d_counts, sizeof(int) * nimg) != cudaSuccess) {
        cudaFree(d_lines);
        return HL_OUT_OF_MEM;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int saved_rows = h->win_rows_override, saved_thr = h->threads_override;
    const int saved_graph = h->batch_graph;
    h->batch_graph = 0;
    hl_tune_entry bst = {0, 0, 3.0e38f};
    int n = 0, rc = HL_NO_ERROR;
    for (int ti = 0; ti < 2 && rc == HL_NO_ERROR; ti++) {
        for (int ri = 0; ri < 5 && rc == HL_NO_ERROR; ri++) {
            const int rows = std::min(row_cand[ri], maxr);
            if (ri < 4 && row_cand[ri] >= maxr)
                continue;   /* the last candidate covers it */
            h->win_rows_override = rows;
            h->threads_override = thr_cand[ti];
            /* warm-up (plans, allocates), then three timed calls */
            rc = batch_run(h, imgs, nimg, thresholds, K, d_lines, d_counts, s);
            if (rc != HL_NO_ERROR)
                break;
            cudaEventRecord(e0, s);
            for (int r = 0; r < 3 && rc == HL_NO_ERROR; r++)
                rc = batch_run(h, imgs, nimg, thresholds, K, d_lines, d_counts, s);
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = HL_CUDA_ERROR;
                break;
            }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms /= 3.0f;
            hl_tune_entry te = {rows, thr_cand[ti], ms};
            if (tried && n < max_tried)
                tried[n] = te;
            n++;
            if (ms < bst.ms)
                bst = te;
        }
    }
    int st = 0;
    if (rc == HL_NO_ERROR && batch_last_status(h, &st, s) == HL_NO_ERROR && st != 0)
        rc = HL_CUDA_ERROR;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_lines);
    cudaFree(d_counts);
    h->batch_graph = saved_graph;
    if (rc != HL_NO_ERROR || bst.threads == 0) {
        h->win_rows_override = saved_rows;
        h->threads_override = saved_thr;
        return rc != HL_NO_ERROR ? rc : HL_CUDA_ERROR;
    }
    h->win_rows_override = bst.window_rows;
    h->threads_override = bst.threads;
    *best = bst;
    if (ntried)
        *ntried = n;
    return HL_NO_ERROR;
}

/* ==================================================================== */
/* Proposal-guided batched path                                          */
/* ==================================================================== */

struct hl_prop_ws {
    __nv_bfloat16 *d_occ;          /* [n][256][256] */
    size_t cap_occ;
    unsigned char *d_tab;          /* pool descriptors + head geometries */
    size_t cap_tab;
    unsigned char *h_tab;
    size_t cap_htab;
    int4 *d_win;
    size_t cap_win;
    int *d_cnt;                    /* [0] windows [1] status [2..3] votes [4] cells */
    int *d_fb;                     /* per-image fall-back flags */
    size_t cap_fb;
    int *h_fb;                     /* pinned copy */
    size_t cap_hfb;
    hl_line *d_fb_lines;           /* plain results of the fall-back set */
    size_t cap_fb_lines;
    int *d_fb_counts;
    size_t cap_fb_counts;
    int *d_map;                    /* fall-back slot -> image */
    size_t cap_map;
};

static void prop_free(hl_handle *h)
{
    hl_prop_ws *p = h->pw;
    if (!p)
        return;
    void *dp[] = {p->d_occ, p->d_tab, p->d_win, p->d_cnt, p->d_fb, p->d_fb_lines,
                  p->d_fb_counts, p->d_map};
    for (void *q : dp)
        if (q)
            cudaFree(q);
    if (p->h_tab)
        cudaFreeHost(p->h_tab);
    if (p->h_fb)
        cudaFreeHost(p->h_fb);
    delete p;
    h->pw = nullptr;
}

/* copy fall-back results (slot q -> image map[q]) into the outputs */
__global__ void hl_scatter_results_kernel(const hl_line *src_lines,
                                          const int *src_counts, const int *map,
                                          int nmap, int K, hl_line *dst_lines,
                                          int *dst_counts)
{
    for (int q = blockIdx.x; q < nmap; q += gridDim.x) {
        const int i = map[q];
        if (i < 0)
            continue;
        for (int j = threadIdx.x; j < K; j += blockDim.x)
            dst_lines[(size_t)i * K + j] = src_lines[(size_t)q * K + j];
        if (threadIdx.x == 0)
            dst_counts[i] = src_counts[q];
    }
}

extern "C" int hl_proposal_batch(hl_handle *h, hl_net *net,
                                 const hl_image_desc *imgs, int nimg,
                                 const int *thresholds, int linesmax,
                                 const hl_proposal_opts *opts,
                                 hl_line *lines_dev, int *counts_dev,
                                 hl_proposal_stats *stats, void *stream)
{
    if (!h || !net || !imgs || !opts || !counts_dev)
        return HL_NULL_POINTER;
    if (linesmax > 0 && !lines_dev)
        return HL_NULL_POINTER;
    if (nimg <= 0 || nimg > 0xffff || !(opts->p_cut > 0.0f && opts->p_cut < 1.0f) ||
        opts->max_props < 0 || opts->dilate_rho < 0 || opts->dilate_theta < 0 ||
        opts->judge_every < 0 || opts->top_m < 0 || opts->top_m > 1024 ||
        !(opts->p_conf >= 0.0f && opts->p_conf < 1.0f))
        return HL_INVALID_DATA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int K = std::max(linesmax, 0);
    if (!h->bw) {
        h->bw = new (std::nothrow) hl_batch_ws();
        if (!h->bw)
            return HL_OUT_OF_MEM;
    }
    if (!h->pw) {
        h->pw = new (std::nothrow) hl_prop_ws();
        if (!h->pw)
            return HL_OUT_OF_MEM;
    }
    hl_batch_ws *b = h->bw;
    hl_prop_ws *pw = h->pw;
    std::vector<hl_roi> rois((size_t)nimg);
    int rc;
    for (int i = 0; i < nimg; i++)
        if ((rc = roi_of(&imgs[i], &rois[i])) != HL_NO_ERROR)
            return rc;
    if ((rc = batch_plan(h, b, imgs, nimg, thresholds, K, lines_dev, counts_dev,
                         rois.data())) != HL_NO_ERROR)
        return rc;
    h->last_batch = 1;

    /* pool descriptors and head geometries (host), window capacity */
    const size_t off_geo = align16(sizeof(hl_pool_img) * nimg);
    const size_t tab = off_geo + sizeof(hl_head_geom) * nimg;
    size_t max_bins = 1;
    int nk_fast = 0;
    std::vector<char> force((size_t)nimg, 0);
    if (!b->tab_event) {
        CK(cudaEventCreateWithFlags(&b->tab_read, cudaEventDisableTiming));
        b->tab_event = 1;
    }
    CK(cudaEventSynchronize(b->tab_read));   /* pw->h_tab reuse */
    if ((rc = grow_host(&pw->h_tab, &pw->cap_htab, tab)) != HL_NO_ERROR ||
        (rc = grow((void **)&pw->d_tab, &pw->cap_tab, tab)) != HL_NO_ERROR ||
        (rc = grow((void **)&pw->d_occ, &pw->cap_occ,
                   sizeof(__nv_bfloat16) * 256 * 256 * (size_t)nimg)) != HL_NO_ERROR ||
        (rc = grow((void **)&pw->d_fb, &pw->cap_fb, sizeof(int) * nimg)) != HL_NO_ERROR ||
        (rc = grow_host((unsigned char **)&pw->h_fb, &pw->cap_hfb, sizeof(int) * nimg)) !=
            HL_NO_ERROR)
        return rc;
    if (!pw->d_cnt)
        CK(cudaMalloc(&pw->d_cnt, 8 * sizeof(int)));
    hl_pool_img *pi = reinterpret_cast<hl_pool_img *>(pw->h_tab);
    hl_head_geom *hg = reinterpret_cast<hl_head_geom *>(pw->h_tab + off_geo);
    for (int i = 0; i < nimg; i++) {
        const int w = rois[i].w, hh = rois[i].h;
        const int f = std::max(1, (std::max(w, hh) + 255) / 256);
        pi[i].base = rois[i].base;
        pi[i].pitch = rois[i].pitch;
        pi[i].w = w;
        pi[i].h = hh;
        pi[i].factor = f;
        pi[i].pad = 0;
        hg[i].cell = (float)(4 * f);
        hg[i].rho_min = (float)b->rho_min[i];
        hg[i].inv_rw = (float)HL_COARSE_R / (float)b->R[i];
        hg[i].qh = ((hh + f - 1) / f + 3) / 4;
        hg[i].qw = ((w + f - 1) / f + 3) / 4;
        hg[i].pad = 0;
        const int nk = (h->T + HL_COARSE_T - 1) / HL_COARSE_T + 2;
        const int nj = HL_WIN_RUN * ((b->R[i] + HL_COARSE_R - 1) / HL_COARSE_R) + 2;
        /* columns of nj rows plus a dump row; the branch-free vote for at
         * most 6 or 10 thetas writes that many columns */
        nk_fast = nk <= 6 ? 6 : (nk <= 10 ? 10 : 0);
        max_bins = std::max(max_bins, (size_t)std::max(nk, nk_fast) * (size_t)(nj + 1));
        const int ntiles = ((w + HL_TILE_W - 1) / HL_TILE_W) * ((hh + HL_TILE_H - 1) / HL_TILE_H);
        if (ntiles > HL_WIN_MAXTILES)
            force[i] = 1;
    }
    if (max_bins * sizeof(int) > 200u * 1024u)
        return HL_OP_OVERFLOW;
    const int cap_win = nimg * (std::max(1, opts->max_props) + std::max(0, opts->top_m) + 64) *
                        (2 * opts->dilate_rho + 1) * (2 * opts->dilate_theta + 1);
    if ((rc = grow((void **)&pw->d_win, &pw->cap_win, sizeof(int4) * (size_t)cap_win)) !=
        HL_NO_ERROR)
        return rc;

    /* device work: compaction, pooling, network, selection, windows, finalize */
    unsigned char *dt = b->d_tab;
    CK(cudaMemsetAsync(pw->d_cnt, 0, 8 * sizeof(int), s));
    CK(cudaMemcpyAsync(pw->d_tab, pw->h_tab, tab, cudaMemcpyHostToDevice, s));
    if ((rc = batch_enqueue_compact(h, b, nimg, s)) != HL_NO_ERROR)
        return rc;
    CK(hl_launch_pool(reinterpret_cast<const hl_pool_img *>(pw->d_tab), nimg, 256, pw->d_occ, s));
    const float *logits = nullptr;
    if ((rc = hl_net_run(net, pw->d_occ,
                         reinterpret_cast<const hl_head_geom *>(pw->d_tab + off_geo), nimg,
                         &logits, s)) != HL_NO_ERROR)
        return rc;
    hl_select_args sa;
    memset(&sa, 0, sizeof(sa));
    sa.logits = logits;
    sa.zcut = logf(opts->p_cut / (1.0f - opts->p_cut));
    sa.max_props = opts->max_props;
    sa.top_m = opts->top_m;
    sa.dil_t = opts->dilate_theta;
    sa.dil_r = opts->dilate_rho;
    sa.force_fallback = 0;
    sa.nms = opts->nms ? 1 : 0;
    sa.use_conf = opts->p_conf > 0.0f ? 1 : 0;
    sa.zconf = sa.use_conf ? logf(opts->p_conf / (1.0f - opts->p_conf)) : 0.0f;
    sa.fallback = pw->d_fb;
    sa.win = pw->d_win;
    sa.nwin = pw->d_cnt + 0;
    sa.ncells = pw->d_cnt + 4;
    sa.cap = cap_win;
    sa.status = pw->d_cnt + 1;
    CK(hl_launch_select(&sa, nimg, s));
    hl_window_args wa;
    memset(&wa, 0, sizeof(wa));
    wa.win = pw->d_win;
    wa.nwin = pw->d_cnt + 0;
    wa.cap = cap_win;
    wa.vimgs = reinterpret_cast<const hl_vote_img *>(dt + b->off_vimg);
    wa.pimgs = reinterpret_cast<const hl_peak_img *>(dt + b->off_pimg);
    wa.cosv = h->d_cos;
    wa.sinv = h->d_sin;
    wa.T = h->T;
    wa.irho = (float)(1.0 / h->p.derho);
    wa.votes = stats ? reinterpret_cast<unsigned long long *>(pw->d_cnt + 2) : nullptr;
    wa.status = pw->d_cnt + 1;
    wa.nk_fast = nk_fast;
    CK(hl_launch_window_vote(&wa, (int)max_bins, std::max(1, h->sms) * 6, s));
    if ((rc = batch_enqueue_finalize(h, b, nimg, K, s)) != HL_NO_ERROR)
        return rc;
    CK(cudaEventRecord(b->tab_read, s));

    /* fall-back and judged images run the plain method */
    int st_host[5] = {0, 0, 0, 0, 0};
    CK(cudaMemcpyAsync(pw->h_fb, pw->d_fb, sizeof(int) * nimg, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(st_host, pw->d_cnt, sizeof(st_host), cudaMemcpyDeviceToHost, s));
    int nst = 0;
    if ((rc = hl_net_status(net, &nst, s)) != HL_NO_ERROR)
        return rc;
    CK(cudaStreamSynchronize(s));
    if (st_host[1] != 0 || nst != 0)
        return HL_CUDA_ERROR;
    std::vector<int> sub, sub_fb;    /* images to run plain; is it a fall-back */
    for (int i = 0; i < nimg; i++) {
        const bool fb = pw->h_fb[i] != 0 || force[i];
        const bool judge = !fb && opts->judge_every > 0 && i % opts->judge_every == 0;
        if (fb || judge) {
            sub.push_back(i);
            sub_fb.push_back(fb ? 1 : 0);
        }
    }
    int n_fb = 0, judged = 0, jl = 0, jf = 0, n_conf = 0;
    for (int i = 0; i < nimg; i++)
        n_conf += pw->h_fb[i] == 2;
    if (!sub.empty()) {
        const int ns = (int)sub.size();
        std::vector<hl_image_desc> sd((size_t)ns);
        std::vector<int> sthr((size_t)ns);
        for (int q = 0; q < ns; q++) {
            sd[q] = imgs[sub[q]];
            sthr[q] = thresholds ? thresholds[sub[q]] : h->p.threshold;
        }
        const size_t KK = (size_t)std::max(K, 1);
        if ((rc = grow((void **)&pw->d_fb_lines, &pw->cap_fb_lines,
                       sizeof(hl_line) * KK * ns)) != HL_NO_ERROR ||
            (rc = grow((void **)&pw->d_fb_counts, &pw->cap_fb_counts, sizeof(int) * ns)) !=
                HL_NO_ERROR ||
            (rc = grow((void **)&pw->d_map, &pw->cap_map, sizeof(int) * ns)) != HL_NO_ERROR)
            return rc;
        if ((rc = batch_run_ws(h, &h->bw_fb, sd.data(), ns, sthr.data(), K, pw->d_fb_lines,
                               pw->d_fb_counts, s)) != HL_NO_ERROR)
            return rc;
        h->last_batch = 1;
        std::vector<int> map((size_t)ns, -1);
        for (int q = 0; q < ns; q++)
            if (sub_fb[q]) {
                map[q] = sub[q];
                n_fb++;
            }
        CK(cudaMemcpyAsync(pw->d_map, map.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        if (n_fb > 0) {
            hl_scatter_results_kernel<<<std::min(ns, 1024), 128, 0, s>>>(
                pw->d_fb_lines, pw->d_fb_counts, pw->d_map, ns, K, lines_dev, counts_dev);
            CK(cudaGetLastError());
        }
        int fst = 0;
        CK(cudaMemcpyAsync(&fst, h->bw_fb->d_cnt + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
        /* recall of the judged images: plain lines found by the proposals */
        std::vector<hl_line> pl, pp;
        std::vector<int> pc, qc;
        const int nj = ns - n_fb;
        if (nj > 0 && K > 0) {
            pl.resize(KK * ns);
            pc.resize(ns);
            pp.resize(KK * nimg);
            qc.resize(nimg);
            CK(cudaMemcpyAsync(pl.data(), pw->d_fb_lines, sizeof(hl_line) * KK * ns,
                               cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(pc.data(), pw->d_fb_counts, sizeof(int) * ns,
                               cudaMemcpyDeviceToHost, s));
            for (int q = 0; q < ns; q++) {
                if (sub_fb[q])
                    continue;
                const int i = sub[q];
                CK(cudaMemcpyAsync(pp.data() + KK * i, lines_dev + (size_t)i * K,
                                   sizeof(hl_line) * K, cudaMemcpyDeviceToHost, s));
                CK(cudaMemcpyAsync(qc.data() + i, counts_dev + i, sizeof(int),
                                   cudaMemcpyDeviceToHost, s));
            }
        }
        CK(cudaStreamSynchronize(s));
        if (fst != 0)
            return HL_CUDA_ERROR;
        if (nj > 0 && K > 0) {
            for (int q = 0; q < ns; q++) {
                if (sub_fb[q])
                    continue;
                const int i = sub[q];
                judged++;
                const int np = std::min(pc[q], K), nq = std::min(qc[i], K);
                jl += np;
                for (int a = 0; a < np; a++) {
                    const hl_line &L = pl[KK * q + a];
                    for (int c = 0; c < nq; c++) {
                        const hl_line &M = pp[KK * i + c];
                        if (M.angle == L.angle && M.distance == L.distance &&
                            M.votes == L.votes) {
                            jf++;
                            break;
                        }
                    }
                }
            }
        }
    }
    if (stats) {
        stats->fallback = n_fb;
        stats->windows = std::min(st_host[0], cap_win);
        stats->judged = judged;
        stats->judged_lines = jl;
        stats->judged_found = jf;
        stats->fallback_conf = n_conf;
        unsigned long long v = 0;
        memcpy(&v, &st_host[2], sizeof(v));
        stats->votes = (long long)v;
        stats->cells = st_host[4];
        stats->pad = 0;
    }
    return HL_NO_ERROR;
}

/* ---- HoughCircle (include/hl_circle.h) ---------------------------------- */

static int circle_prepare(hl_handle *h, const hl_image_desc *img, const hl_circle_params *p,
                          hl_roi *roi, hl_geom *g)
{
    if (!h || !img || !p)
        return HL_NULL_POINTER;
    if (p->radius_min < 0 || p->radius_max < p->radius_min || p->radius_max >= 65536 ||
        p->threshold < 0 || !(p->dist_thres == p->dist_thres))
        return HL_INVALID_DATA;
    int rc = roi_of(img, roi);
    if (rc != HL_NO_ERROR)
        return rc;
    if ((rc = hl_geometry(h, roi->w, roi->h, g)) != HL_NO_ERROR)
        return rc;
    return ensure_image(h, *g, roi->w, roi->h);
}

/* the compaction, then one tile-kernel launch: the accumulator written to acc
 * ([nr][h][w]) when it is given, the local maxima appended to the handle's
 * candidate keys when peaks is set */
static int circle_run(hl_handle *h, const hl_roi &roi, const hl_geom &g,
                      const hl_circle_params *p, int32_t *acc, bool peaks, cudaStream_t s)
{
    const int nr = p->radius_max - p->radius_min + 1;
    hl_circle_tile_args ta;
    memset(&ta, 0, sizeof(ta));
    ta.ntx = (roi.w + HL_CIRCLE_TW - 1) / HL_CIRCLE_TW;
    ta.nty = (roi.h + HL_CIRCLE_TH - 1) / HL_CIRCLE_TH;
    if ((long long)ta.ntx * ta.nty * nr > 0x7fffffffLL)
        return HL_OP_OVERFLOW;   /* more CTAs than one launch takes */
    int rc = launch_compaction(h, roi, g, s);
    if (rc != HL_NO_ERROR)
        return rc;
    ta.pts = reinterpret_cast<const float2 *>(h->d_pts);
    ta.tile_off = h->d_tile_off;
    ta.ctiles_x = g.tiles_x;
    ta.ctiles_y = g.tiles_y;
    ta.w = roi.w;
    ta.h = roi.h;
    ta.rmin = p->radius_min;
    ta.nr = nr;
    ta.acc = acc;
    ta.threshold = p->threshold;
    if (peaks) {
        ta.keys = h->d_ckeys;
        ta.ncand = h->d_ccnt;
        ta.cap = HL_CIRCLE_MAXCAND;
        ta.status = h->d_ccnt + 1;
    }
    CK(hl_launch_circle_tiles(&ta, s));
    return HL_NO_ERROR;
}

extern "C" int hl_circle_accumulator(hl_handle *h, const hl_image_desc *img,
                                     const hl_circle_params *p, int32_t *acc_dev,
                                     void *stream)
{
    if (!acc_dev)
        return HL_NULL_POINTER;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    hl_roi roi;
    hl_geom g;
    int rc = circle_prepare(h, img, p, &roi, &g);
    if (rc != HL_NO_ERROR)
        return rc;
    if ((rc = circle_run(h, roi, g, p, acc_dev, false, s)) != HL_NO_ERROR)
        return rc;
    /* the compaction's status word (a bounded wait that gave up) */
    int st = 0;
    CK(cudaMemcpyAsync(&st, h->d_counters + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (st != 0) {
        reset_counters(h, s);
        return HL_CUDA_ERROR;
    }
    return HL_NO_ERROR;
}

extern "C" int hl_circles(hl_handle *h, const hl_image_desc *img, const hl_circle_params *p,
                          int *circlemax, hl_circle *out, void *stream)
{
    if (!circlemax)
        return HL_NULL_POINTER;
    if (*circlemax > 0 && !out)
        return HL_NULL_POINTER;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    hl_roi roi;
    hl_geom g;
    int rc = circle_prepare(h, img, p, &roi, &g);
    if (rc != HL_NO_ERROR)
        return rc;
    const int nr = p->radius_max - p->radius_min + 1;
    const size_t cells = (size_t)nr * roi.w * roi.h;
    if (cells >= (size_t)0xffffffffu)
        return HL_OP_OVERFLOW;   /* the candidate key holds a 32-bit index */
    const int cm = std::max(*circlemax, 0);
    const size_t rbytes = sizeof(hl_result_hdr) + sizeof(hl_circle) * (size_t)std::max(cm, 1);
    if (!h->d_ckeys) {
        CK(cudaMalloc(&h->d_ckeys, sizeof(unsigned long long) * HL_CIRCLE_MAXCAND));
        CK(cudaMalloc(&h->d_ccnt, 2 * sizeof(int)));
        CK(cudaMemset(h->d_ccnt, 0, 2 * sizeof(int)));
    }
    /* results: header + room for circlemax circles, pinned mirror */
    static const size_t kResCap = sizeof(hl_result_hdr) + sizeof(hl_circle) * 4096;
    if (rbytes > kResCap)
        return HL_INVALID_DATA;
    if (!h->d_cres) {
        CK(cudaMalloc(&h->d_cres, kResCap));
        CK(cudaMallocHost(&h->h_cres, kResCap + sizeof(int)));
    }
    if ((rc = circle_run(h, roi, g, p, nullptr, true, s)) != HL_NO_ERROR)
        return rc;
    hl_circle_final_args fa;
    fa.imgs = nullptr;
    fa.keys = h->d_ckeys;
    fa.ncand = h->d_ccnt;
    fa.w = roi.w;
    fa.h = roi.h;
    fa.rmin = p->radius_min;
    fa.dist_thres = p->dist_thres;
    fa.r_thres = p->r_thres;
    fa.circlemax = cm;
    fa.roi_x = img->roi_x1;
    fa.roi_y = img->roi_y1;
    fa.out = reinterpret_cast<hl_circle *>(h->d_cres + sizeof(hl_result_hdr));
    fa.hdr = reinterpret_cast<hl_result_hdr *>(h->d_cres);
    fa.status = h->d_ccnt + 1;
    CK(hl_launch_circle_final(&fa, 1, s));
    /* the results and the compaction's status word */
    int *cstat = reinterpret_cast<int *>(h->h_cres + kResCap);
    CK(cudaMemcpyAsync(h->h_cres, h->d_cres, rbytes, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(cstat, h->d_counters + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const hl_result_hdr *hdr = reinterpret_cast<const hl_result_hdr *>(h->h_cres);
    if (*cstat != 0) {
        reset_counters(h, s);
        return HL_CUDA_ERROR;
    }
    if (hdr->status != 0)
        return (hdr->status & HL_ST_CAND_OVERFLOW) ? HL_OP_OVERFLOW : HL_CUDA_ERROR;
    if (hdr->count > 0)
        memcpy(out, h->h_cres + sizeof(hl_result_hdr), sizeof(hl_circle) * (size_t)hdr->count);
    *circlemax = hdr->count;
    return HL_NO_ERROR;
}

/* ---- HoughCircle batches -------------------------------------------------- */

struct hl_cb_ws {
    float2 *d_pts;
    size_t cap_pts;
    int *d_toff;
    size_t cap_toff;
    unsigned long long *d_state;
    size_t cap_state;
    unsigned char *d_tab;
    size_t cap_tab;
    unsigned char *h_tab;
    size_t cap_htab;
    unsigned long long *d_keys;
    size_t cap_keys;
    int *d_cnt;
    size_t cap_cnt;
    unsigned char *d_res;
    size_t cap_res;
    unsigned char *h_res;
    size_t cap_hres;
};

static void circle_batch_free(hl_handle *h)
{
    hl_cb_ws *c = h->cb;
    if (!c)
        return;
    void *dp[] = {c->d_pts, c->d_toff, c->d_state, c->d_tab, c->d_keys, c->d_cnt, c->d_res};
    for (void *q : dp)
        if (q)
            cudaFree(q);
    if (c->h_tab)
        cudaFreeHost(c->h_tab);
    if (c->h_res)
        cudaFreeHost(c->h_res);
    delete c;
    h->cb = nullptr;
}

/* Circles of many ROIs (of one image or several) in one pipeline: one
 * compaction over every ROI (the batch form of the compaction kernel, each
 * ROI its own point region and tile offsets), one tile launch over every
 * ROI's (tile, radius) CTAs, one tail CTA per ROI, one copy of the results. */
extern "C" int hl_circles_batch(hl_handle *h, const hl_image_desc *imgs, int nimg,
                                const hl_circle_params *p, int circlemax, hl_circle *out,
                                int *counts, void *stream)
{
    if (!h || !p || !counts || (nimg > 0 && !imgs) || (nimg > 0 && circlemax > 0 && !out))
        return HL_NULL_POINTER;
    if (nimg < 0 || circlemax < 0 || circlemax > HL_CIRCLE_MAXCAND)
        return HL_INVALID_DATA;
    if (p->radius_min < 0 || p->radius_max < p->radius_min || p->radius_max >= 65536 ||
        p->threshold < 0 || !(p->dist_thres == p->dist_thres))
        return HL_INVALID_DATA;
    if (nimg == 0)
        return HL_NO_ERROR;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int nr = p->radius_max - p->radius_min + 1;
    std::vector<hl_roi> rois((size_t)nimg);
    std::vector<hl_geom> gs((size_t)nimg);
    std::vector<long long> pts_base((size_t)nimg);
    std::vector<int> tile_base((size_t)nimg), group_base((size_t)nimg), cta_base((size_t)nimg);
    std::vector<int> group_img;
    long long pts = 0, ctas = 0, tiles = 0, groups = 0;
    for (int i = 0; i < nimg; i++) {
        int rc = roi_of(&imgs[i], &rois[i]);
        if (rc != HL_NO_ERROR)
            return rc;
        if ((rc = hl_geometry(h, rois[i].w, rois[i].h, &gs[i])) != HL_NO_ERROR)
            return rc;
        if ((size_t)nr * rois[i].w * rois[i].h >= (size_t)0xffffffffu)
            return HL_OP_OVERFLOW;   /* the candidate key holds a 32-bit index */
        const int nt = gs[i].tiles_x * gs[i].tiles_y;
        const int ng = (nt + HL_COMPACT_GROUP - 1) / HL_COMPACT_GROUP;
        tile_base[i] = (int)tiles;
        group_base[i] = (int)groups;
        for (int q = 0; q < ng; q++)
            group_img.push_back(i);
        tiles += nt + 1;   /* the ROI's tile offsets and its end */
        groups += ng;
        /* every pixel and one pad per tile, even so each region starts on
         * 16 bytes */
        pts_base[i] = pts;
        pts += ((long long)rois[i].w * rois[i].h + nt + 16 + 1) & ~1LL;
        const long long ntx = (rois[i].w + HL_CIRCLE_TW - 1) / HL_CIRCLE_TW;
        const long long nty = (rois[i].h + HL_CIRCLE_TH - 1) / HL_CIRCLE_TH;
        cta_base[i] = (int)std::min(ctas, (long long)0x7fffffff);
        ctas += ntx * nty * nr;
        if (ctas > 0x7fffffffLL || tiles > 0x7fffffffLL || groups > 0x7fffffffLL)
            return HL_OP_OVERFLOW;
    }
    if (!h->cb && !(h->cb = new (std::nothrow) hl_cb_ws()))
        return HL_OUT_OF_MEM;
    hl_cb_ws *c = h->cb;
    const size_t rstride =
        align16(sizeof(hl_result_hdr) + sizeof(hl_circle) * (size_t)std::max(circlemax, 1));
    const size_t off_cimg = 0;
    const size_t off_gimg = align16(sizeof(hl_compact_img) * (size_t)nimg);
    const size_t off_circ = align16(off_gimg + sizeof(int) * (size_t)groups);
    const size_t tab_bytes = align16(off_circ + sizeof(hl_circle_img) * (size_t)nimg);
    const size_t ncnt = 4 + 2 * (size_t)nimg;   /* ticket, count, status, pad, per ROI */
    int rc;
    if ((rc = grow((void **)&c->d_pts, &c->cap_pts, sizeof(float2) * (size_t)pts)) != HL_NO_ERROR ||
        (rc = grow((void **)&c->d_toff, &c->cap_toff, sizeof(int) * (size_t)tiles)) != HL_NO_ERROR ||
        (rc = grow((void **)&c->d_state, &c->cap_state,
                   sizeof(unsigned long long) * (size_t)(groups + 1))) != HL_NO_ERROR ||
        (rc = grow((void **)&c->d_tab, &c->cap_tab, tab_bytes)) != HL_NO_ERROR ||
        (rc = grow_host(&c->h_tab, &c->cap_htab, tab_bytes)) != HL_NO_ERROR ||
        (rc = grow((void **)&c->d_keys, &c->cap_keys,
                   sizeof(unsigned long long) * HL_CIRCLE_MAXCAND * (size_t)nimg)) != HL_NO_ERROR ||
        (rc = grow((void **)&c->d_cnt, &c->cap_cnt, sizeof(int) * ncnt)) != HL_NO_ERROR ||
        (rc = grow((void **)&c->d_res, &c->cap_res, rstride * (size_t)nimg)) != HL_NO_ERROR ||
        (rc = grow_host(&c->h_res, &c->cap_hres, rstride * (size_t)nimg + 16)) != HL_NO_ERROR)
        return rc;
    hl_compact_img *ci = reinterpret_cast<hl_compact_img *>(c->h_tab + off_cimg);
    hl_circle_img *im = reinterpret_cast<hl_circle_img *>(c->h_tab + off_circ);
    for (int i = 0; i < nimg; i++) {
        const hl_geom &g = gs[i];
        const int nt = g.tiles_x * g.tiles_y;
        ci[i].roi = rois[i];
        ci[i].tiles_x = g.tiles_x;
        ci[i].ntiles = nt;
        ci[i].tile_base = tile_base[i];
        ci[i].group_base = group_base[i];
        ci[i].ngroups = (nt + HL_COMPACT_GROUP - 1) / HL_COMPACT_GROUP;
        ci[i].pad = 0;
        ci[i].pts_base = pts_base[i];
        im[i].pts = c->d_pts + pts_base[i];
        im[i].tile_off = c->d_toff + tile_base[i];
        im[i].ctiles_x = g.tiles_x;
        im[i].ctiles_y = g.tiles_y;
        im[i].w = rois[i].w;
        im[i].h = rois[i].h;
        im[i].ntx = (rois[i].w + HL_CIRCLE_TW - 1) / HL_CIRCLE_TW;
        im[i].nty = (rois[i].h + HL_CIRCLE_TH - 1) / HL_CIRCLE_TH;
        im[i].roi_x = imgs[i].roi_x1;
        im[i].roi_y = imgs[i].roi_y1;
        im[i].cta_base = cta_base[i];
        im[i].pad = 0;
        im[i].keys = c->d_keys + (size_t)HL_CIRCLE_MAXCAND * i;
        im[i].ncand = c->d_cnt + 4 + 2 * i;
        im[i].hdr = reinterpret_cast<hl_result_hdr *>(c->d_res + rstride * i);
        im[i].out = reinterpret_cast<hl_circle *>(c->d_res + rstride * i + sizeof(hl_result_hdr));
    }
    memcpy(c->h_tab + off_gimg, group_img.data(), sizeof(int) * group_img.size());
    unsigned char *dt = c->d_tab;
    CK(cudaMemsetAsync(c->d_cnt, 0, sizeof(int) * ncnt, s));
    CK(cudaMemsetAsync(c->d_state, 0, sizeof(unsigned long long) * (size_t)(groups + 1), s));
    CK(cudaMemcpyAsync(dt, c->h_tab, tab_bytes, cudaMemcpyHostToDevice, s));
    hl_compact_args ca;
    memset(&ca, 0, sizeof(ca));
    ca.imgs = reinterpret_cast<const hl_compact_img *>(dt + off_cimg);
    ca.group_img = reinterpret_cast<const int *>(dt + off_gimg);
    ca.nimg = nimg;
    ca.ngroups = (int)groups;
    ca.tile_state = c->d_state;
    ca.ticket = reinterpret_cast<unsigned *>(c->d_cnt + 0);
    ca.ticket_base = 0;
    ca.epoch = 1;
    ca.pts = nullptr;
    ca.pts_f2 = c->d_pts;
    ca.tile_off = c->d_toff;
    ca.count = c->d_cnt + 1;
    ca.status = c->d_cnt + 2;
    CK(hl_launch_compact(&ca, s));
    hl_circle_tile_args ta;
    memset(&ta, 0, sizeof(ta));
    ta.imgs = reinterpret_cast<const hl_circle_img *>(dt + off_circ);
    ta.nimg = nimg;
    ta.nctas = (int)ctas;
    ta.rmin = p->radius_min;
    ta.nr = nr;
    ta.acc = nullptr;
    ta.threshold = p->threshold;
    ta.cap = HL_CIRCLE_MAXCAND;
    CK(hl_launch_circle_tiles(&ta, s));
    hl_circle_final_args fa;
    memset(&fa, 0, sizeof(fa));
    fa.imgs = reinterpret_cast<const hl_circle_img *>(dt + off_circ);
    fa.rmin = p->radius_min;
    fa.dist_thres = p->dist_thres;
    fa.r_thres = p->r_thres;
    fa.circlemax = circlemax;
    CK(hl_launch_circle_final(&fa, nimg, s));
    int *cstat = reinterpret_cast<int *>(c->h_res + rstride * (size_t)nimg);
    CK(cudaMemcpyAsync(c->h_res, c->d_res, rstride * (size_t)nimg, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(cstat, c->d_cnt + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (*cstat != 0)
        return HL_CUDA_ERROR;
    rc = HL_NO_ERROR;
    for (int i = 0; i < nimg; i++) {
        const hl_result_hdr *hdr =
            reinterpret_cast<const hl_result_hdr *>(c->h_res + rstride * (size_t)i);
        if (hdr->status != 0) {
            counts[i] = 0;
            if (rc == HL_NO_ERROR)
                rc = (hdr->status & HL_ST_CAND_OVERFLOW) ? HL_OP_OVERFLOW : HL_CUDA_ERROR;
            continue;
        }
        counts[i] = hdr->count;
        if (hdr->count > 0)
            memcpy(out + (size_t)circlemax * i, c->h_res + rstride * (size_t)i + sizeof(hl_result_hdr),
                   sizeof(hl_circle) * (size_t)hdr->count);
    }
    return rc;
}

