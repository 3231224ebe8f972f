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
 *   Both kernels also take a batch (a table of images): the tile launch covers
 *       every image's (tile, radius) CTAs, the tail runs one CTA per image.
 *   hl_circle_final_kernel -- one CTA: rank sort (votes descending, index
 *       ascending: the deviation from the reference's shear sort is only the
 *       order of equal votes), decode (:632-657), the greedy merge of
 *       _recalCirParam (:809-871) on one warp, output with the ROI offset.
 */
#include "hl_internal.h"

#define FULL 0xffffffffu

/* ---- vote + local maxima ------------------------------------------------- */

/* local cell (x, y) is image cell (x + tx0 - CT_OX, y + ty0 - 1): the
 * interior starts on a 16-byte boundary of every row, the apron is the column
 * before and after it and the rows above and below */
#define CT_OX 4
#define CT_AW (HL_CIRCLE_TW + 8)
#define CT_AH (HL_CIRCLE_TH + 2)
#define CT_CELLS (CT_AH * CT_AW)
#define CT_THREADS 1024
#define CT_WARPS (CT_THREADS / 32)
#define CT_ROWS 256   /* compaction-tile rows of the halo taken per pass */

#ifndef CT_SEG
#define CT_SEG 4            /* lanes (segments of the walk) per point */
#endif
#define CT_QN (32 / CT_SEG) /* points per walk */
struct CtSeg {
    int nloop;                        /* steps of the longest segment */
    int len[CT_SEG];                  /* steps of each segment */
    int x[CT_SEG], y[CT_SEG], d[CT_SEG];   /* the state where it starts */
};

struct CircleTileSmem {
    int cnt[CT_CELLS];        /* the tile and its apron, row-major */
    int pre[CT_ROWS + 1];     /* points of the halo rows before each row */
    int start[CT_ROWS];       /* first point of each halo row */
    int red[CT_WARPS];
    unsigned char rank_lane[CT_WARPS][32];   /* lane of the k-th queued point */
    int2 left[CT_WARPS * 32];                /* the warps' last, partial queues */
    int nleft;
    int nextb;                               /* next candidate batch of the pass */
    CtSeg seg;                              /* the segments of this CTA's walk */
};

/* one vote at the shared-memory word addr when p holds: a predicated
 * red.shared, so a warp's eight octant votes of a step issue without a
 * branch around each */
__device__ __forceinline__ void ct_red(unsigned addr, bool p)
{
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %1, 0;\n\t@q red.shared.add.u32 [%0], 1;\n\t}"
                 :: "r"(addr), "r"((int)p) : "memory");
}

/* A lane's votes: its point (x0, y0) walks (part of) the midpoint circle of
 * radius r (okano_3_0/HoughCircle.cu:214-243) and votes the octant points
 * that fall in [0, xw) x [0, yh); pbase is the shared address of that
 * region's origin.  The warp's lanes share r, so the loop is uniform. */
/* The walk of one radius split into CT_SEG segments on CT_SEG lanes.  The
 * midpoint recurrence (x, y, d) depends on r only, so the state where each
 * segment starts is the same for every point: lane l walks segment l / CT_QN
 * of point l % CT_QN.  A walk covers CT_QN points in about 1 / CT_SEG of the
 * steps of a whole walk, so the CTA's walks are CT_SEG times as many and as
 * short, and the warps finish closer together. */
__device__ __forceinline__ void ct_walk_seg(int x0, int y0, const CtSeg &hw, int seg,
                                            int xw, int yh, unsigned pbase)
{
    int x = hw.x[seg], y = hw.y[seg], d = hw.d[seg];
    const int mylen = hw.len[seg], nloop = hw.nloop;
    for (int it = 0; it < nloop; it++) {
        const bool act = it < mylen;
        const int xa = x0 + x, xb = x0 - x, xc = x0 + y, xd = x0 - y;
        const int ya = y0 + y, yb = y0 - y, yc = y0 + x, yd = y0 - x;
        const bool fxa = act && (unsigned)xa < (unsigned)xw;
        const bool fxb = act && (unsigned)xb < (unsigned)xw;
        const bool fxc = act && (unsigned)xc < (unsigned)xw;
        const bool fxd = act && (unsigned)xd < (unsigned)xw;
        const bool fya = (unsigned)ya < (unsigned)yh, fyb = (unsigned)yb < (unsigned)yh;
        const bool fyc = (unsigned)yc < (unsigned)yh, fyd = (unsigned)yd < (unsigned)yh;
        const unsigned ra = pbase + 4u * (unsigned)(ya * CT_AW);
        const unsigned rb = pbase + 4u * (unsigned)(yb * CT_AW);
        const unsigned rc = pbase + 4u * (unsigned)(yc * CT_AW);
        const unsigned rd = pbase + 4u * (unsigned)(yd * CT_AW);
        /* okano_3_0/HoughCircle.cu:227-234 */
        ct_red(ra + 4u * (unsigned)xa, fxa && fya);
        ct_red(rb + 4u * (unsigned)xa, fxa && fyb);
        ct_red(ra + 4u * (unsigned)xb, fxb && fya);
        ct_red(rb + 4u * (unsigned)xb, fxb && fyb);
        ct_red(rc + 4u * (unsigned)xc, fxc && fyc);
        ct_red(rd + 4u * (unsigned)xc, fxc && fyd);
        ct_red(rc + 4u * (unsigned)xd, fxd && fyc);
        ct_red(rd + 4u * (unsigned)xd, fxd && fyd);
        const bool up = d < y;
        d += up ? 4 * x + 6 : 4 * (x - y) + 10;
        y -= up ? 0 : 1;
        x++;
    }
}

/* a point no vote of which lands in the counted cells (an idle lane): every
 * coordinate stays negative for radii below 65536, and y * CT_AW fits an int */
#define CT_NOWHERE (-(1 << 20))

__global__ void __launch_bounds__(CT_THREADS, 1)
hl_circle_tile_kernel(hl_circle_tile_args a0)
{
    extern __shared__ __align__(16) unsigned char ct_raw[];
    CircleTileSmem &sm = *reinterpret_cast<CircleTileSmem *>(ct_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    {
        int4 *c4 = reinterpret_cast<int4 *>(sm.cnt);
        for (int i = tid; i < CT_CELLS / 4; i += CT_THREADS)
            c4[i] = make_int4(0, 0, 0, 0);
    }
    if (tid == 0)
        sm.nleft = 0;
    hl_pdl_begin();
    hl_circle_tile_args a = a0;
    unsigned bid = blockIdx.x;
    if (a0.imgs) {
        /* a batch: the image whose CTA range holds this CTA */
        int lo = 0, hi = a0.nimg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((unsigned)a0.imgs[mid].cta_base <= bid)
                lo = mid;
            else
                hi = mid - 1;
        }
        const hl_circle_img im = a0.imgs[lo];
        a.pts = im.pts;
        a.tile_off = im.tile_off;
        a.ctiles_x = im.ctiles_x;
        a.ctiles_y = im.ctiles_y;
        a.w = im.w;
        a.h = im.h;
        a.ntx = im.ntx;
        a.nty = im.nty;
        a.keys = im.keys;
        a.ncand = im.ncand;
        a.status = im.ncand + 1;
        bid -= (unsigned)im.cta_base;
    }
    const int ntile = a.ntx * a.nty;
    const int z = a.nr - 1 - (int)(bid / (unsigned)ntile);
    const int tile = (int)(bid % (unsigned)ntile);
    const int r = a.rmin + z;
    const int tx0 = (tile % a.ntx) * HL_CIRCLE_TW, ty0 = (tile / a.ntx) * HL_CIRCLE_TH;
    /* counted cells, image coordinates: the tile and its apron within the ROI */
    const int cx0 = max(tx0 - 1, 0), cy0 = max(ty0 - 1, 0);
    const int cx1 = min(tx0 + HL_CIRCLE_TW + 1, a.w), cy1 = min(ty0 + HL_CIRCLE_TH + 1, a.h);
    if (tid == 0 && r > 0) {
        /* the midpoint recurrence of radius r (okano_3_0/HoughCircle.cu:
         * 214-243): its step count, and the state where each segment starts */
        int x = 0, y = r, d = 3 - 2 * r, n = 0;
        while (x < y) {
            const bool up = d < y;
            d += up ? 4 * x + 6 : 4 * (x - y) + 10;
            y -= up ? 0 : 1;
            x++;
            n++;
        }
        /* segment k: steps [k n / CT_SEG, (k + 1) n / CT_SEG) */
        CtSeg hw;
        x = 0;
        y = r;
        d = 3 - 2 * r;
        int step = 0;
        for (int k = 0; k < CT_SEG; k++) {
            const int b0 = k * n / CT_SEG, b1 = (k + 1) * n / CT_SEG;
            while (step < b0) {
                const bool up = d < y;
                d += up ? 4 * x + 6 : 4 * (x - y) + 10;
                y -= up ? 0 : 1;
                x++;
                step++;
            }
            hw.x[k] = x;
            hw.y[k] = y;
            hw.d[k] = d;
            hw.len[k] = b1 - b0;
        }
        hw.nloop = 0;
        for (int k = 0; k < CT_SEG; k++)
            hw.nloop = max(hw.nloop, hw.len[k]);
        sm.seg = hw;
    }
    __syncthreads();
    if (r > 0) {
        const int xlo = cx0 - tx0 + CT_OX, xw = cx1 - cx0;
        const int ylo = cy0 - ty0 + 1, yh = cy1 - cy0;
        const unsigned pbase = (unsigned)__cvta_generic_to_shared(sm.cnt) +
                               4u * (unsigned)(ylo * CT_AW + xlo);
        /* the halo: points within r of the counted cells */
        const int hx0 = max(cx0 - r, 0), hx1 = min(cx1 - 1 + r, a.w - 1);
        const int hy0 = max(cy0 - r, 0), hy1 = min(cy1 - 1 + r, a.h - 1);
        const int ctx0 = hx0 / HL_TILE_W, ctx1 = hx1 / HL_TILE_W;
        const int cty0 = hy0 / HL_TILE_H, cty1 = hy1 / HL_TILE_H;
        int qx = CT_NOWHERE, qy = CT_NOWHERE, qn = 0;   /* the warp's queue: lanes < qn */
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
            if (tid == 0) {
                sm.pre[0] = 0;
                sm.nextb = 0;
            }
            __syncthreads();
            const int total = sm.pre[nrow];
            /* a warp takes the next 32 consecutive candidates (a shared
             * counter: a warp busy walking takes fewer) and queues those
             * inside the halo, one per lane; a full queue walks its 32
             * circles at once */
            while (true) {
                int ib = 0;
                if (lane == 0)
                    ib = atomicAdd(&sm.nextb, 32);
                ib = __shfl_sync(FULL, ib, 0);
                if (ib >= total)
                    break;
                const int i = ib + lane;
                int cx = CT_NOWHERE, cy = CT_NOWHERE;
                bool ok = false;
                if (i < total) {
                    int lo = 0, hi = nrow - 1;   /* the row k with pre[k] <= i < pre[k + 1] */
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (sm.pre[mid] <= i)
                            lo = mid;
                        else
                            hi = mid - 1;
                    }
                    const float2 pt = a.pts[sm.start[lo] + (i - sm.pre[lo])];
                    /* the compaction's sentinel of an odd tile is 1e30 */
                    if (pt.x < 1.0e29f) {
                        const int px = (int)pt.x, py = (int)pt.y;
                        ok = px >= hx0 && px <= hx1 && py >= hy0 && py <= hy1;
                        cx = px - tx0 + CT_OX - xlo;
                        cy = py - ty0 + 1 - ylo;
                    }
                }
                const unsigned vm = __ballot_sync(FULL, ok);
                const int nv = __popc(vm);
                if (ok)
                    sm.rank_lane[warp][__popc(vm & ((1u << lane) - 1u))] = (unsigned char)lane;
                __syncwarp();
                /* the queue is lanes [0, CT_QN); slots [qn, qn + take) take
                 * the next ranks, and a full queue walks its circles at once,
                 * CT_SEG lanes a point */
                for (int done = 0; done < nv;) {
                    const int take = min(CT_QN - qn, nv - done);
                    const bool fill = lane >= qn && lane < qn + take;
                    const int src = fill ? sm.rank_lane[warp][done + lane - qn] : lane;
                    const int nx = __shfl_sync(FULL, cx, src), ny = __shfl_sync(FULL, cy, src);
                    if (fill) {
                        qx = nx;
                        qy = ny;
                    }
                    qn += take;
                    done += take;
                    if (qn == CT_QN) {
                        const int px = __shfl_sync(FULL, qx, lane % CT_QN);
                        const int py = __shfl_sync(FULL, qy, lane % CT_QN);
                        ct_walk_seg(px, py, sm.seg, lane / CT_QN, xw, yh, pbase);
                        qx = CT_NOWHERE;
                        qy = CT_NOWHERE;
                        qn = 0;
                    }
                }
                __syncwarp();   /* rank_lane is rewritten by the next batch */
            }
            __syncthreads();   /* before the next pass rewrites pre / start */
        }
        /* the partial queues left in every warp are pooled and walked CT_QN
         * points at a time, not as up to 32 part-empty walks */
        if (lane < qn)
            sm.left[atomicAdd(&sm.nleft, 1)] = make_int2(qx, qy);
        __syncthreads();
        const int nl = sm.nleft;
        for (int b0 = warp * CT_QN; b0 < nl; b0 += CT_WARPS * CT_QN) {
            const int k = b0 + lane % CT_QN;
            const int2 q = k < nl ? sm.left[k] : make_int2(CT_NOWHERE, CT_NOWHERE);
            ct_walk_seg(q.x, q.y, sm.seg, lane / CT_QN, xw, yh, pbase);
        }
    }
    __syncthreads();
    /* the interior: written out and/or its local maxima taken (cells
     * outside the ROI were never counted: their zeros are the reference's
     * border).  A warp takes whole rows, a lane four cells of one 16-byte
     * load; the neighbour tests run only where one of the four is above the
     * threshold. */
    const int iw = min(HL_CIRCLE_TW, a.w - tx0), ih = min(HL_CIRCLE_TH, a.h - ty0);
    const size_t zrow = (size_t)z * a.h;
    for (int row = warp; row < ih; row += CT_WARPS) {
        const int *prow = sm.cnt + (row + 1) * CT_AW + CT_OX;
        for (int c0 = 0; c0 < iw; c0 += 128) {
            const int col = c0 + 4 * lane;
            int4 q = make_int4(0, 0, 0, 0);
            if (col < iw)
                q = *reinterpret_cast<const int4 *>(prow + col);
            if (a.acc) {
                int32_t *g = a.acc + (zrow + ty0 + row) * a.w + tx0 + col;
                const int vv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int e = 0; e < 4; e++)
                    if (col + e < iw)
                        g[e] = vv[e];
            }
            if (!a.keys)
                continue;
            const int m = max(max(q.x, q.y), max(q.z, q.w));
            if (!__any_sync(FULL, m > a.threshold))
                continue;
            const int vv[4] = {q.x, q.y, q.z, q.w};
            unsigned mine = 0;
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int *p = prow + col + e;
                const int v = vv[e];
                if (col + e < iw && v > a.threshold && v > p[-1] && v >= p[1] &&
                    v > p[-CT_AW] && v >= p[CT_AW])
                    mine |= 1u << e;
            }
            const int cnt = __popc(mine);
            int pos = cnt ? atomicAdd(a.ncand, cnt) : 0;
#pragma unroll
            for (int e = 0; e < 4; e++) {
                if (mine & (1u << e)) {
                    const unsigned idx =
                        (unsigned)((zrow + ty0 + row) * a.w + tx0 + col + e);
                    if (pos < a.cap)
                        a.keys[pos] = ((unsigned long long)(unsigned)vv[e] << 32) |
                                      (unsigned)(~idx);
                    else
                        atomicOr(a.status, HL_ST_CAND_OVERFLOW);
                    pos++;
                }
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

__global__ void __launch_bounds__(1024, 1)
hl_circle_final_kernel(hl_circle_final_args a0)
{
    extern __shared__ __align__(16) unsigned char c_raw[];
    CircleSmem &sm = *reinterpret_cast<CircleSmem *>(c_raw);
    hl_pdl_begin();
    const hl_circle_final_args &a = a0;
    /* a batch: this CTA's image */
    const hl_circle_img *im = a.imgs ? a.imgs + blockIdx.x : nullptr;
    const unsigned long long *keys = im ? im->keys : a.keys;
    int *const ncandp = im ? im->ncand : a.ncand;
    int *const statusp = im ? im->ncand + 1 : a.status;
    const int W = im ? im->w : a.w, H = im ? im->h : a.h;
    const int roi_x = im ? im->roi_x : a.roi_x, roi_y = im ? im->roi_y : a.roi_y;
    hl_circle *const outp = im ? im->out : a.out;
    hl_result_hdr *const hdrp = im ? im->hdr : a.hdr;
    const int tid = threadIdx.x;
    const int ncand = *ncandp;
    /* past the key buffer the call fails (OP_OVERFLOW): nothing to rank */
    const int n = ncand > HL_CIRCLE_MAXCAND ? 0 : ncand;
    for (int i = tid; i < n; i += blockDim.x)
        sm.keys[i] = keys[i];
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
    const long long plane = (long long)W * H;
    for (int i = tid; i < n; i += blockDim.x) {
        const unsigned long long k = sm.sorted[i];
        const long long idx = (long long)(unsigned)(~(unsigned)(k & 0xffffffffu));
        const long long z = idx / plane, t = idx - z * plane;
        sm.cir[i] = make_int4((int)(t % W), (int)(t / W), (int)z + a.rmin, (int)(k >> 32));
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
                o.a = c.x + roi_x;
                o.b = c.y + roi_y;
                o.radius = c.z;
                o.votes = c.w;
                outp[k++] = o;
            }
        }
        hdrp->count = k;
        hdrp->ncand = ncand;
        int st = *statusp;
        if (ncand > HL_CIRCLE_MAXCAND)
            st |= HL_ST_CAND_OVERFLOW;
        hdrp->status = st;
        *statusp = 0;
        *ncandp = 0;
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
    const long long grid = a->imgs ? (long long)a->nctas : (long long)a->ntx * a->nty * a->nr;
    if (grid <= 0 || grid > 0x7fffffffLL)
        return cudaErrorInvalidConfiguration;
    return hl_launch_pdl(hl_circle_tile_kernel, dim3((unsigned)grid), dim3(CT_THREADS), smem, s,
                         false, *a);
}

cudaError_t hl_launch_circle_final(const hl_circle_final_args *a, int nimg, cudaStream_t s)
{
    const size_t smem = sizeof(CircleSmem);
    cudaError_t e = cudaFuncSetAttribute(hl_circle_final_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    if (nimg < 1)
        return cudaErrorInvalidValue;
    return hl_launch_pdl(hl_circle_final_kernel, dim3((unsigned)nimg), dim3(1024), smem, s,
                         false, *a);
}
