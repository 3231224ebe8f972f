/*
 * hl_circle.cu -- HoughCircle on the HoughLine engine (the image path of
 * HoughCircle::houghcircle, okano_3_0/HoughCircle.cu:927-1165): the edge
 * pixels come from the same compaction, votes are counted in (radius, row,
 * column) accumulator tiles in shared memory, the local maxima taken in the
 * same pass, then a one-CTA tail.
 *
 *   hl_circle_tile_kernel -- one CTA per (accumulator tile, radius), largest
 *       radius first.  The CTA counts its tile and a one-cell apron: every
 *       edge point within the radius of them (read from the compaction tiles
 *       that overlap that halo) walks the reference's midpoint circle
 *       (okano_3_0/HoughCircle.cu:187-245: x = 0, y = r, d = 3 - 2r; while
 *       x < y ...; eight octant points a step, the points on the axes twice)
 *       and adds shared-memory atomics for the points inside the counted
 *       cells; votes outside the ROI are dropped, as the reference drops
 *       them.  The whole sum of a cell is then in shared memory, so the
 *       interior is written out (the accumulator entry point) and/or its
 *       local maxima taken (okano_3_0/HoughCircle.cu:321-370: v above the
 *       threshold, above the left and upper neighbours and at least the
 *       right and lower ones, zero outside the ROI) with the apron as the
 *       neighbours; the keys (votes << 32 | ~index) are appended with one
 *       atomic per warp.  The accumulator never goes to HBM on the circle
 *       path.
 *   hl_circle_final_kernel -- one CTA: rank sort (votes descending, index
 *       ascending: the deviation from the reference's shear sort is only the
 *       order of equal votes), decode (:632-657), the greedy merge of
 *       _recalCirParam (:809-871) on one warp, output with the ROI offset.
 */
#include "hl_internal.h"

#define FULL 0xffffffffu

/* ---- vote + local maxima ------------------------------------------------- */

#define CT_AW (HL_CIRCLE_TW + 2)
#define CT_AH (HL_CIRCLE_TH + 2)
#define CT_THREADS 512
#define CT_ROWS 256   /* compaction-tile rows of the halo taken per pass */

struct CircleTileSmem {
    int cnt[CT_AH * CT_AW];   /* the tile and its apron, row-major */
    int pre[CT_ROWS + 1];     /* points of the halo rows before each row */
    int start[CT_ROWS];       /* first point of each halo row */
    int red[CT_THREADS / 32];
};

/* one vote at local cell (x, y) when it lies in [xlo, xhi) x [ylo, yhi) */
__device__ __forceinline__ void ct_vote(int *cnt, int x, int y, int xlo, int xw, int ylo,
                                        int yh)
{
    if ((unsigned)(x - xlo) < (unsigned)xw && (unsigned)(y - ylo) < (unsigned)yh)
        atomicAdd(cnt + y * CT_AW + x, 1);
}

__global__ void __launch_bounds__(CT_THREADS, 2)
hl_circle_tile_kernel(hl_circle_tile_args a)
{
    extern __shared__ __align__(16) unsigned char ct_raw[];
    CircleTileSmem &sm = *reinterpret_cast<CircleTileSmem *>(ct_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ntile = a.ntx * a.nty;
    const int z = a.nr - 1 - (int)(blockIdx.x / (unsigned)ntile);
    const int tile = (int)(blockIdx.x % (unsigned)ntile);
    const int r = a.rmin + z;
    const int tx0 = (tile % a.ntx) * HL_CIRCLE_TW, ty0 = (tile / a.ntx) * HL_CIRCLE_TH;
    /* counted cells, image coordinates: the tile and its apron within the ROI;
     * local cell (x, y) is image cell (x + tx0 - 1, y + ty0 - 1) */
    const int cx0 = max(tx0 - 1, 0), cy0 = max(ty0 - 1, 0);
    const int cx1 = min(tx0 + HL_CIRCLE_TW + 1, a.w), cy1 = min(ty0 + HL_CIRCLE_TH + 1, a.h);
    {
        int4 *c4 = reinterpret_cast<int4 *>(sm.cnt);
        for (int i = tid; i < CT_AH * CT_AW / 4; i += CT_THREADS)
            c4[i] = make_int4(0, 0, 0, 0);
    }
    hl_pdl_begin();
    __syncthreads();
    if (r > 0) {
        const int xlo = cx0 - (tx0 - 1), xw = cx1 - cx0;
        const int ylo = cy0 - (ty0 - 1), yh = cy1 - cy0;
        /* the halo: points within r of the counted cells */
        const int hx0 = max(cx0 - r, 0), hx1 = min(cx1 - 1 + r, a.w - 1);
        const int hy0 = max(cy0 - r, 0), hy1 = min(cy1 - 1 + r, a.h - 1);
        const int ctx0 = hx0 / HL_TILE_W, ctx1 = hx1 / HL_TILE_W;
        const int cty0 = hy0 / HL_TILE_H, cty1 = hy1 / HL_TILE_H;
        for (int row0 = cty0; row0 <= cty1; row0 += CT_ROWS) {
            const int nrow = min(CT_ROWS, cty1 - row0 + 1);
            /* the halo's compaction tiles of one row are consecutive, and so
             * are their points */
            int len = 0;
            if (tid < nrow) {
                const int t = (row0 + tid) * a.ctiles_x;
                const int s0 = a.tile_off[t + ctx0];
                len = a.tile_off[t + ctx1 + 1] - s0;
                sm.start[tid] = s0;
            }
            int v = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(FULL, v, o);
                if (lane >= o)
                    v += t;
            }
            if (lane == 31 && warp < CT_ROWS / 32)
                sm.red[warp] = v;
            __syncthreads();
            if (tid < CT_ROWS) {
                int off = 0;
                for (int k = 0; k < warp; k++)
                    off += sm.red[k];
                sm.pre[tid + 1] = off + v;
            }
            if (tid == 0)
                sm.pre[0] = 0;
            __syncthreads();
            const int total = sm.pre[nrow];
            for (int i = tid; i < total; i += CT_THREADS) {
                int lo = 0, hi = nrow - 1;   /* the row k with pre[k] <= i < pre[k + 1] */
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (sm.pre[mid] <= i)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                const float2 pt = a.pts[sm.start[lo] + (i - sm.pre[lo])];
                if (!(pt.x < 1.0e29f))
                    continue;   /* the compaction's sentinel of an odd tile */
                const int px = (int)pt.x, py = (int)pt.y;
                if (px < hx0 || px > hx1 || py < hy0 || py > hy1)
                    continue;
                const int x0 = px - (tx0 - 1), y0 = py - (ty0 - 1);
                int x = 0, y = r, d = 3 - 2 * r;
                while (x < y) {
                    ct_vote(sm.cnt, x0 + x, y0 + y, xlo, xw, ylo, yh);
                    ct_vote(sm.cnt, x0 + x, y0 - y, xlo, xw, ylo, yh);
                    ct_vote(sm.cnt, x0 - x, y0 + y, xlo, xw, ylo, yh);
                    ct_vote(sm.cnt, x0 - x, y0 - y, xlo, xw, ylo, yh);
                    ct_vote(sm.cnt, x0 + y, y0 + x, xlo, xw, ylo, yh);
                    ct_vote(sm.cnt, x0 + y, y0 - x, xlo, xw, ylo, yh);
                    ct_vote(sm.cnt, x0 - y, y0 + x, xlo, xw, ylo, yh);
                    ct_vote(sm.cnt, x0 - y, y0 - x, xlo, xw, ylo, yh);
                    if (d < y)
                        d += 4 * x + 6;
                    else {
                        d += 4 * (x - y) + 10;
                        y--;
                    }
                    x++;
                }
            }
            __syncthreads();   /* before the next pass rewrites pre / start */
        }
    }
    /* the interior: written out and/or its local maxima taken (cells
     * outside the ROI were never counted: their zeros are the reference's
     * border) */
    const int iw = min(HL_CIRCLE_TW, a.w - tx0), ih = min(HL_CIRCLE_TH, a.h - ty0);
    const size_t zrow = (size_t)z * a.h;
    for (int c = tid; c < HL_CIRCLE_TW * HL_CIRCLE_TH; c += CT_THREADS) {
        const int row = c / HL_CIRCLE_TW, col = c - row * HL_CIRCLE_TW;
        const bool in = col < iw && row < ih;
        const int *p = sm.cnt + (row + 1) * CT_AW + (col + 1);
        const int v = in ? p[0] : 0;
        if (a.acc && in)
            a.acc[(zrow + ty0 + row) * a.w + tx0 + col] = v;
        if (a.keys) {
            const bool is = in && v > a.threshold && v > p[-1] && v >= p[1] &&
                            v > p[-CT_AW] && v >= p[CT_AW];
            const unsigned b = __ballot_sync(FULL, is);
            if (!b)
                continue;
            int pos = 0;
            if (lane == 0)
                pos = atomicAdd(a.ncand, __popc(b));
            pos = __shfl_sync(FULL, pos, 0) + __popc(b & ((1u << lane) - 1u));
            if (is) {
                const unsigned idx = (unsigned)((zrow + ty0 + row) * a.w + tx0 + col);
                if (pos < a.cap)
                    a.keys[pos] = ((unsigned long long)(unsigned)v << 32) | (unsigned)(~idx);
                else
                    atomicOr(a.status, HL_ST_CAND_OVERFLOW);
            }
        }
    }
}

/* ---- tail ---------------------------------------------------------------- */

struct CircleSmem {
    unsigned long long keys[HL_CIRCLE_MAXCAND];
    unsigned long long sorted[HL_CIRCLE_MAXCAND];
    int4 cir[HL_CIRCLE_MAXCAND];   /* a, b, radius, votes */
    int misc[4];
};

/* is circle j close to circle i (the test of okano_3_0/HoughCircle.cu:
 * 834-841: centre distance squared in float, radius difference in int) */
__device__ __forceinline__ bool circle_close(int4 ci, int4 cj, float d2, int r_thres)
{
    const int da = ci.x - cj.x, db = ci.y - cj.y;
    const float dist = __fadd_rn(__fmul_rn((float)da, (float)da), (float)(db * db));
    return dist < d2 && abs(ci.z - cj.z) < r_thres;
}

__global__ void __launch_bounds__(1024)
hl_circle_final_kernel(hl_circle_final_args a)
{
    extern __shared__ __align__(16) unsigned char c_raw[];
    CircleSmem &sm = *reinterpret_cast<CircleSmem *>(c_raw);
    hl_pdl_begin();
    const int tid = threadIdx.x;
    const int ncand = *a.ncand;
    /* past the key buffer the call fails (OP_OVERFLOW): nothing to rank */
    const int n = ncand > HL_CIRCLE_MAXCAND ? 0 : ncand;
    for (int i = tid; i < n; i += blockDim.x)
        sm.keys[i] = a.keys[i];
    __syncthreads();
    /* rank sort, descending (keys are unique: the index is part of them) */
    for (int i = tid; i < n; i += blockDim.x) {
        const unsigned long long ki = sm.keys[i];
        int rank = 0;
        for (int j = 0; j < n; j++)
            rank += sm.keys[j] > ki;
        sm.sorted[rank] = ki;
    }
    __syncthreads();
    const long long plane = (long long)a.w * a.h;
    for (int i = tid; i < n; i += blockDim.x) {
        const unsigned long long k = sm.sorted[i];
        const long long idx = (long long)(unsigned)(~(unsigned)(k & 0xffffffffu));
        const long long z = idx / plane, t = idx - z * plane;
        sm.cir[i] = make_int4((int)(t % a.w), (int)(t / a.w), (int)z + a.rmin, (int)(k >> 32));
    }
    __syncthreads();
    if (tid < 32) {
        /* _recalCirParam: for each circle i in rank order (passed over when
         * its votes or radius are zero), every later circle j within the
         * thresholds of i's current parameters is averaged into i and
         * zeroed.  32 j are tested at a time; only the first hit is applied,
         * then the rest of the chunk is tested again against the new i. */
        const int lane = tid;
        const float d2 = __fmul_rn(a.dist_thres, a.dist_thres);
        int circlenum = 0;
        for (int i = 0; i < n; i++) {
            int4 ci = sm.cir[i];
            if (ci.w == 0 || ci.z == 0)
                continue;
            for (int j0 = i + 1; j0 < n; j0 += 32) {
                int from = 0;   /* lanes below have been applied or missed */
                while (true) {
                    const int j = j0 + lane;
                    const bool hit = lane >= from && j < n &&
                                     circle_close(ci, sm.cir[j], d2, a.r_thres);
                    const unsigned b = __ballot_sync(FULL, hit);
                    if (!b)
                        break;
                    const int f = __ffs(b) - 1;
                    const int4 cj = sm.cir[j0 + f];
                    ci = make_int4((ci.x + cj.x) / 2, (ci.y + cj.y) / 2, (ci.z + cj.z) / 2,
                                   ci.w + cj.w);
                    __syncwarp();
                    if (lane == 0) {
                        sm.cir[j0 + f] = make_int4(0, 0, 0, 0);
                        sm.cir[i] = ci;
                    }
                    __syncwarp();
                    from = f + 1;
                }
            }
            circlenum++;
        }
        if (lane == 0)
            sm.misc[0] = circlenum;
    }
    __syncthreads();
    if (tid == 0) {
        int cm = min(sm.misc[0], a.circlemax);
        int k = 0;
        for (int i = 0; i < n && k < cm; i++) {
            const int4 c = sm.cir[i];
            if (c.w != 0) {
                hl_circle o;
                o.a = c.x + a.roi_x;
                o.b = c.y + a.roi_y;
                o.radius = c.z;
                o.votes = c.w;
                a.out[k++] = o;
            }
        }
        a.hdr->count = k;
        a.hdr->ncand = ncand;
        int st = *a.status;
        if (ncand > HL_CIRCLE_MAXCAND)
            st |= HL_ST_CAND_OVERFLOW;
        a.hdr->status = st;
        *a.status = 0;
        *a.ncand = 0;
    }
}

/* ---- launchers ----------------------------------------------------------- */

cudaError_t hl_launch_circle_tiles(const hl_circle_tile_args *a, cudaStream_t s)
{
    const size_t smem = sizeof(CircleTileSmem);
    cudaError_t e = cudaFuncSetAttribute(hl_circle_tile_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    const long long grid = (long long)a->ntx * a->nty * a->nr;
    if (grid <= 0 || grid > 0x7fffffffLL)
        return cudaErrorInvalidConfiguration;
    return hl_launch_pdl(hl_circle_tile_kernel, dim3((unsigned)grid), dim3(CT_THREADS), smem, s,
                         false, *a);
}

cudaError_t hl_launch_circle_final(const hl_circle_final_args *a, cudaStream_t s)
{
    const size_t smem = sizeof(CircleSmem);
    cudaError_t e = cudaFuncSetAttribute(hl_circle_final_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    return hl_launch_pdl(hl_circle_final_kernel, dim3(1), dim3(1024), smem, s, false, *a);
}
