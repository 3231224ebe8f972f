/*
 * hl_stage_a.cu -- cos/sin table and stage (a): edge-pixel compaction.
 *
 * Compaction replaces the flag / ScanArray / scatter chain of
 * ImgConvert::imgConvertToCst (okano_3_0/ImgConvert.cu:142-353,
 * okano_3_0/ScanArray.cu:1351+) with ONE pass: every CTA reads a group of
 * four 128 x 32 tiles with 16-byte vector loads (all four issued before any
 * is used), counts their 255-pixels with one packed block scan, obtains the
 * group's exclusive prefix by decoupled look-back over its predecessors'
 * published aggregates, and scatters packed coordinates.  The predicate is
 * the vote kernel's `pixel == 255` (okano_3_0/HoughLine.cu:125), not
 * ImgConvert's `>= 128`.
 *
 * HBM-bound: each image byte is read once (w*h bytes) and each edge point is
 * written once (4 bytes).
 */
#include <algorithm>

#include "hl_internal.h"

#define FULL 0xffffffffu

/* theta_k = (float)(k * detheta) and CUDA's cosf/sinf of it: the values the
 * reference vote kernel computes inline (okano_3_0/HoughLine.cu:115-119). */
__global__ void hl_trig_kernel(float *cosv, float *sinv, int T, int Tp,
                               double detheta)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Tp)
        return;
    if (k < T) {
        float th = (float)(k * detheta);
        cosv[k] = cosf(th);
        sinv[k] = sinf(th);
    } else {
        cosv[k] = 0.0f;
        sinv[k] = 0.0f;
    }
}

cudaError_t hl_launch_trig(float *cosv, float *sinv, int T, int Tp,
                           double detheta, cudaStream_t s)
{
    hl_trig_kernel<<<(Tp + 127) / 128, 128, 0, s>>>(cosv, sinv, T, Tp, detheta);
    return cudaGetLastError();
}

/* 4-bit mask of the bytes of w equal to 0xFF (bit i = byte i). */
__device__ __forceinline__ uint32_t eq255x4(uint32_t w)
{
    uint32_t m = __vcmpeq4(w, 0xffffffffu) & 0x80808080u;
    return (m * 0x00204081u) >> 28;
}

/* The same mask by exact SWAR arithmetic: a byte of ~w is zero exactly when
 * the byte of w is 0xFF; (b & 0x7F) + 0x7F sets the high bit of every
 * nonzero low part with no carry between bytes, OR b keeps the rest. */
__device__ __forceinline__ uint32_t ff_nibble(uint32_t w)
{
    const uint32_t t = ~w;
    const uint32_t nz = (((t & 0x7f7f7f7fu) + 0x7f7f7f7fu) | t) & 0x80808080u;
    return ((~nz & 0x80808080u) * 0x00204081u) >> 28;
}

/* Look-back state word: epoch (30 bits) | flag (2 bits) | value (32 bits).
 * flag 1 = aggregate of this tile only, 2 = inclusive prefix. */
#define LB_AGG 1ull
#define LB_PRE 2ull
#define LB_SPIN_LIMIT (1 << 18)

__device__ __forceinline__ unsigned long long lb_pack(unsigned epoch,
                                                      unsigned long long flag,
                                                      unsigned value)
{
    return ((unsigned long long)epoch << 34) | (flag << 32) | value;
}

__device__ __forceinline__ void lb_store(unsigned long long *p,
                                         unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v)
                 : "memory");
}

__device__ __forceinline__ unsigned long long lb_load(
    const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];"
                 : "=l"(v)
                 : "l"(p)
                 : "memory");
    return v;
}

/* Warp-wide decoupled look-back (all 32 lanes of warp 0 call it).  Returns
 * the exclusive prefix of `tile`.  Waits are bounded: past LB_SPIN_LIMIT
 * polls the status word gets HL_ST_LOOKBACK_TIMEOUT and the partial sum is
 * used, so the kernel always ends. */
__device__ int lookback(unsigned long long *state, int tile, int total,
                        unsigned epoch, int *status)
{
    const int lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0)
            lb_store(&state[0], lb_pack(epoch, LB_PRE, (unsigned)total));
        return 0;
    }
    if (lane == 0)
        lb_store(&state[tile], lb_pack(epoch, LB_AGG, (unsigned)total));
    int excl = 0;
    int top = tile - 1;
    int spins = 0;
    while (true) {
        int j = top - lane;
        unsigned long long s = 0;
        unsigned flag;
        if (j >= 0) {
            s = lb_load(&state[j]);
            flag = ((unsigned)(s >> 34) == epoch) ? (unsigned)((s >> 32) & 3u) : 0u;
        } else {
            flag = (unsigned)LB_PRE;   /* before tile 0: prefix 0 */
            s = 0;
        }
        unsigned pmask = __ballot_sync(FULL, flag == LB_PRE);
        unsigned inval = __ballot_sync(FULL, flag == 0);
        int firstp = pmask ? __ffs(pmask) - 1 : 32;
        unsigned need = (firstp >= 31) ? FULL : ((2u << firstp) - 1u);
        if (inval & need) {
            /* give up after LB_SPIN_LIMIT polls, or at once when another
             * tile already gave up, so a failure never cascades into a long
             * chain of timed-out waits */
            bool quit = ++spins > LB_SPIN_LIMIT;
            if (!quit && (spins & 255) == 0)
                quit = (*(volatile int *)status & HL_ST_LOOKBACK_TIMEOUT) != 0;
            quit = __shfl_sync(FULL, quit, 0);
            if (quit) {
                if (lane == 0)
                    atomicOr(status, HL_ST_LOOKBACK_TIMEOUT);
                break;
            }
            __nanosleep(64);
            continue;
        }
        int v = (lane <= firstp && j >= 0) ? (int)(unsigned)(s & 0xffffffffu) : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_xor_sync(FULL, v, o);
        excl += v;
        if (firstp < 32)
            break;
        top -= 32;
    }
    if (lane == 0)
        lb_store(&state[tile], lb_pack(epoch, LB_PRE, (unsigned)(excl + total)));
    return excl;
}

/* Groups a launch may have for the all-predecessor prefix (below). */
#define LB_FULL_MAX 2048

/* Exclusive prefix of group g as the plain sum of every predecessor's own
 * count (all threads of the CTA call it; each group publishes only its count,
 * flag AGG, and never an inclusive prefix).  With every group of a launch
 * resident at once -- a 4096 x 4096 image has 1024 groups -- the chained
 * look-back forwards inclusive prefixes only 32 groups per memory round
 * trip; here a group waits just for its slowest predecessor to publish, and
 * 256 threads read up to 1024 predecessors in one round trip.  Waits are
 * bounded as in lookback(). */
template <int NT>
__device__ int prefix_all(const unsigned long long *state, int g, unsigned epoch,
                          int *status, int *s_red)
{
    const int tid = threadIdx.x;
    int spins = 0;
    while (true) {
        int sum = 0;
        bool bad = false;
        for (int j0 = 0; j0 < g; j0 += 4 * NT) {
            unsigned long long st[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int j = j0 + u * NT + tid;
                st[u] = (j < g) ? lb_load(&state[j]) : 0ull;
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int j = j0 + u * NT + tid;
                if (j < g) {
                    if ((unsigned)(st[u] >> 34) != epoch || ((st[u] >> 32) & 3u) == 0u)
                        bad = true;
                    else
                        sum += (int)(unsigned)(st[u] & 0xffffffffu);
                }
            }
        }
        if (!__syncthreads_or(bad)) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                sum += __shfl_xor_sync(FULL, sum, o);
            if ((tid & 31) == 0)
                s_red[tid >> 5] = sum;
            __syncthreads();
            int t = 0;
            for (int w = 0; w < NT / 32; w++)
                t += s_red[w];
            __syncthreads();
            return t;
        }
        bool quit = ++spins > LB_SPIN_LIMIT;
        if (!quit && (spins & 255) == 0)
            quit = (*(volatile int *)status & HL_ST_LOOKBACK_TIMEOUT) != 0;
        if (__syncthreads_or(quit)) {
            if (tid == 0)
                atomicOr(status, HL_ST_LOOKBACK_TIMEOUT);
            return 0;
        }
        __nanosleep(64);
    }
}

/* Tiles per CTA: one look-back and four 16-byte loads in flight per thread
 * for every 16 KB of image. */
#define CT_GROUP HL_COMPACT_GROUP

__global__ void __launch_bounds__(HL_COMPACT_THREADS, 8)
hl_compact_kernel(hl_compact_args a)
{
    __shared__ int s_grp;
    __shared__ hl_compact_img s_im;
    __shared__ unsigned long long s_wsum[HL_COMPACT_THREADS / 32];
    __shared__ int s_tbase[CT_GROUP];
    __shared__ int s_tcnt[CT_GROUP];
    __shared__ unsigned long long s_tot4;
    __shared__ int s_excl;
    __shared__ int s_red[HL_COMPACT_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ngroups = a.imgs ? a.ngroups : (a.ntiles + CT_GROUP - 1) / CT_GROUP;
    hl_pdl_begin();

    /* Groups are taken in ticket order, so every predecessor of a group is
     * already resident when the group looks back: the waits always end. */
    if (tid == 0) {
        const int g = (int)(atomicAdd(a.ticket, 1u) - a.ticket_base);
        s_grp = g;
        if (!a.imgs) {
            s_im.roi = a.roi;
            s_im.tiles_x = a.tiles_x;
            s_im.ntiles = a.ntiles;
            s_im.tile_base = 0;
            s_im.group_base = 0;
            s_im.ngroups = ngroups;
            s_im.pts_base = 0;
        } else if (g >= 0 && g < ngroups) {
            s_im = a.imgs[a.group_img[g]];
        }
    }
    __syncthreads();
    const int ggrp = s_grp;              /* group in the batch (look-back) */
    if (ggrp < 0 || ggrp >= ngroups)
        return;
    const int grp = ggrp - s_im.group_base;   /* group in its image */
    const int r = tid >> 3, ch = tid & 7;

    /* this thread's 16 pixels of tile q: row ty*32 + r, columns
     * tx*128 + 16*ch .. +15 (recomputed where needed, to keep the live
     * registers low enough for eight CTAs per SM) */
    const int tx0 = (grp * CT_GROUP) % s_im.tiles_x, ty0 = (grp * CT_GROUP) / s_im.tiles_x;
#define CT_TILE_XY(q, xx, yy)                                                  \
    const int xx = ((tx0 + (q)) % s_im.tiles_x) * HL_TILE_W + ch * 16;         \
    const int yy = (ty0 + (tx0 + (q)) / s_im.tiles_x) * HL_TILE_H + r
    /* all loads first */
    uint4 v[CT_GROUP];
#pragma unroll
    for (int q = 0; q < CT_GROUP; q++) {
        CT_TILE_XY(q, xq, yq);
        const bool any = grp * CT_GROUP + q < s_im.ntiles && yq < s_im.roi.h && xq < s_im.roi.w;
        const uint8_t *p = s_im.roi.base + (size_t)yq * (size_t)s_im.roi.pitch + xq;
        const bool vec = any && xq + 16 <= s_im.roi.w && (((uintptr_t)p) & 15u) == 0;
        v[q] = vec ? __ldcs((const uint4 *)p) : make_uint4(0, 0, 0, 0);
    }
    uint32_t m[CT_GROUP];
    unsigned long long cnt4 = 0;   /* four 16-bit counts, tile q in bits 16q */
#pragma unroll
    for (int q = 0; q < CT_GROUP; q++) {
        CT_TILE_XY(q, xq, yq);
        const bool any = grp * CT_GROUP + q < s_im.ntiles && yq < s_im.roi.h && xq < s_im.roi.w;
        const uint8_t *p = s_im.roi.base + (size_t)yq * (size_t)s_im.roi.pitch + xq;
        const bool vec = any && xq + 16 <= s_im.roi.w && (((uintptr_t)p) & 15u) == 0;
        uint32_t mm = 0;
        if (vec) {
            mm = eq255x4(v[q].x) | (eq255x4(v[q].y) << 4) |
                 (eq255x4(v[q].z) << 8) | (eq255x4(v[q].w) << 12);
        } else if (any) {
            const int lim = min(16, s_im.roi.w - xq);
            for (int i = 0; i < lim; i++)
                mm |= (uint32_t)(p[i] == 255) << i;
        }
        m[q] = mm;
        cnt4 |= (unsigned long long)__popc(mm) << (16 * q);
    }
    /* block scan of the packed counts (no field exceeds 4096) */
    unsigned long long incl = cnt4;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o)
            incl += t;
    }
    if (lane == 31)
        s_wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int nw = HL_COMPACT_THREADS / 32;
        const unsigned long long ws = lane < nw ? s_wsum[lane] : 0ull;
        unsigned long long wi = ws;
#pragma unroll
        for (int o = 1; o < nw; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(FULL, wi, o);
            if (lane >= o)
                wi += t;
        }
        const unsigned long long tot4 = __shfl_sync(FULL, wi, nw - 1);
        if (lane < nw)
            s_wsum[lane] = wi - ws;
        /* float2 output: every tile holds an even number of entries (one
         * sentinel pads an odd count), so runs of tiles start and end on
         * 16-byte boundaries */
        const int pad = a.pts_f2 ? 1 : 0;
        int total = 0;
#pragma unroll
        for (int q = 0; q < CT_GROUP; q++) {
            const int cq = (int)((tot4 >> (16 * q)) & 0xffffu);
            total += cq + (cq & pad);
        }
        /* the prefix runs over the image's own groups */
        unsigned long long *st = a.tile_state + s_im.group_base;
        if (s_im.ngroups > LB_FULL_MAX) {
            const int excl = lookback(st, grp, total, a.epoch, a.status);
            if (lane == 0)
                s_excl = excl;
        } else if (lane == 0) {
            lb_store(&st[grp], lb_pack(a.epoch, LB_AGG, (unsigned)total));
        }
        if (lane == 0)
            s_tot4 = tot4;
    }
    __syncthreads();
    if (s_im.ngroups <= LB_FULL_MAX) {
        const int excl = prefix_all<HL_COMPACT_THREADS>(a.tile_state + s_im.group_base, grp,
                                                        a.epoch, a.status, s_red);
        if (tid == 0)
            s_excl = excl;
        __syncthreads();
    }
    {
        const int pad = a.pts_f2 ? 1 : 0;
        const unsigned long long tot4 = s_tot4;
        if (tid == 0) {
            int run = s_excl;
#pragma unroll
            for (int q = 0; q < CT_GROUP; q++) {
                const int tile = grp * CT_GROUP + q;
                const int cq = (int)((tot4 >> (16 * q)) & 0xffffu);
                s_tbase[q] = run;
                s_tcnt[q] = cq;
                if (tile < s_im.ntiles)
                    a.tile_off[s_im.tile_base + tile] = run;
                run += cq + (cq & pad);
            }
            /* the image's end (equal to the next image's start) */
            if (grp == s_im.ngroups - 1)
                a.tile_off[s_im.tile_base + s_im.ntiles] = run;
            if (ggrp == ngroups - 1)
                *a.count = run;
        }
    }
    __syncthreads();
    const unsigned long long ex4 = s_wsum[warp] + incl - cnt4;
#pragma unroll
    for (int q = 0; q < CT_GROUP; q++) {
        CT_TILE_XY(q, xq, yq);
        uint32_t mm = m[q];
        int pos = s_tbase[q] + (int)((ex4 >> (16 * q)) & 0xffffu);
        const uint32_t yy = (uint32_t)yq << 16;
        while (mm) {
            const int bb = __ffs(mm) - 1;
            mm &= mm - 1;
            if (a.pts_f2)
                a.pts_f2[s_im.pts_base + pos] = make_float2((float)(xq + bb), (float)yq);
            else
                a.pts[s_im.pts_base + pos] = (uint32_t)(xq + bb) | yy;
            pos++;
        }
    }
#undef CT_TILE_XY
    /* the sentinel (1e30, 0) never votes inside an accumulator: its rho is
     * 1e30 * cos(theta_k), and cosf of a float angle is never 0 */
    if (a.pts_f2 && tid < CT_GROUP && (s_tcnt[tid] & 1))
        a.pts_f2[s_im.pts_base + s_tbase[tid] + s_tcnt[tid]] = make_float2(1.0e30f, 0.0f);
}

/* Single-image compaction with few, large CTAs: CTA c of nct takes tiles [ntiles c / nct, ntiles (c + 1) / nct) -- at most CP_MAXT --
 * with every one of its 16-byte loads in flight at once, in row order across
 * its tiles; turns them into 16-bit masks of 255-pixels in tile-major order
 * (chunk u = tile * 256 + row * 8 + column chunk, via shared memory), ranks
 * them with one block scan (a thread owns one 128-pixel row of a tile),
 * publishes one count, meets the other CTAs at one grid barrier (a
 * cooperative launch: all CTAs resident) and sums its predecessors' counts
 * in one read -- no polling of every predecessor, whose traffic grows with
 * the square of the CTA count -- then scatters one 16-pixel chunk per
 * thread.  Output as hl_compact_kernel:
 * tile-major, raster order inside a tile, odd float2 tiles padded. */
#define CP_THREADS 1024
#define CP_MAXT 32
#define CP_K (CP_MAXT * 256 / CP_THREADS)

/* tile range of CTA c of nct and the divisor of its row-order load index */
struct CpRange {
    int t0, nt, nu;
    unsigned rowlen, magic;
};
__device__ __forceinline__ CpRange cp_range(const hl_compact_args &a, int c, int nct)
{
    CpRange r;
    r.t0 = (int)((long long)a.ntiles * c / nct);
    r.nt = (int)((long long)a.ntiles * (c + 1) / nct) - r.t0;
    r.nu = r.nt * 256;
    r.rowlen = 8u * (unsigned)r.nt;
    r.magic = 0xffffffffu / r.rowlen + 1u;
    return r;
}

__global__ void __launch_bounds__(CP_THREADS, 1)
hl_compact_persist_kernel(hl_compact_args a, int nct)
{
    __shared__ int s_wsum[CP_THREADS / 32];
    __shared__ int s_tstart[CP_MAXT + 1];   /* point rank at each tile start */
    __shared__ int s_tbase[CP_MAXT];        /* tile offsets within the CTA */
    __shared__ int s_x0[CP_MAXT], s_y0[CP_MAXT];
    __shared__ int s_total, s_excl;
    __shared__ int s_red[CP_THREADS / 32];
    __shared__ __align__(16) unsigned short s_mask[CP_MAXT * 256];
    __shared__ unsigned short s_rowrel[CP_MAXT * 32];   /* row start in its tile */
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    hl_pdl_begin();
    /* a cooperative launch: every CTA is resident, so the CTA index orders
     * the prefix and the grid barrier below always completes */
    const int c = blockIdx.x;
    const CpRange R = cp_range(a, c, nct);
    const int nt = R.nt, nu = R.nu;
    if (tid < nt) {
        s_x0[tid] = ((R.t0 + tid) % a.tiles_x) * HL_TILE_W;
        s_y0[tid] = ((R.t0 + tid) / a.tiles_x) * HL_TILE_H;
    }
    __syncthreads();

    /* loads in row order across the CTA's tiles (load index L = r * 8 nt +
     * tile * 8 + column chunk: a warp reads 512 contiguous bytes of a row),
     * all in flight before any is used; r = L / (8 nt) by a multiply-high,
     * exact for L * 8 nt < 2^32 */
    uint4 v[CP_K];
#pragma unroll
    for (int k = 0; k < CP_K; k++) {
        v[k] = make_uint4(0, 0, 0, 0);
        const int L = tid + k * CP_THREADS;
        if (L < nu) {
            const int r = (int)__umulhi((unsigned)L, R.magic);
            const int rem = L - r * (int)R.rowlen;
            const int x = s_x0[rem >> 3] + (rem & 7) * 16;
            const int y = s_y0[rem >> 3] + r;
            const uint8_t *p = a.roi.base + (size_t)y * (size_t)a.roi.pitch + x;
            if (y < a.roi.h && x + 16 <= a.roi.w && (((uintptr_t)p) & 15u) == 0)
                v[k] = __ldcs((const uint4 *)p);
        }
    }
    /* 16-bit masks of 255-pixels, handed to the tile-major order through
     * shared memory (chunk u = tile * 256 + r * 8 + column chunk) */
#pragma unroll
    for (int k = 0; k < CP_K; k++) {
        const int L = tid + k * CP_THREADS;
        if (L < nu) {
            const int r = (int)__umulhi((unsigned)L, R.magic);
            const int rem = L - r * (int)R.rowlen;
            const int tl = rem >> 3, ch = rem & 7;
            const int x = s_x0[tl] + ch * 16;
            const int y = s_y0[tl] + r;
            uint32_t mm = 0;
            if (y < a.roi.h && x < a.roi.w) {
                const uint8_t *p = a.roi.base + (size_t)y * (size_t)a.roi.pitch + x;
                if (x + 16 <= a.roi.w && (((uintptr_t)p) & 15u) == 0) {
                    mm = ff_nibble(v[k].x) | (ff_nibble(v[k].y) << 4) |
                         (ff_nibble(v[k].z) << 8) | (ff_nibble(v[k].w) << 12);
                } else {
                    const int lim = min(16, a.roi.w - x);
                    for (int i = 0; i < lim; i++)
                        mm |= (uint32_t)(p[i] == 255) << i;
                }
            }
            s_mask[tl * 256 + r * 8 + ch] = (unsigned short)mm;
        }
    }
    __syncthreads();
    /* ranks in tile-major order: thread tid owns row tid % 32 of tile
     * tid / 32 (chunks 8 tid .. 8 tid + 7, one 16-byte shared load); one
     * block scan of the rows' counts */
    const bool owner = tid * 8 < nu;
    int cnt = 0;
    if (owner) {
        const uint4 q = reinterpret_cast<const uint4 *>(s_mask)[tid];
        cnt = __popc(q.x) + __popc(q.y) + __popc(q.z) + __popc(q.w);
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o)
            incl += t;
    }
    if (lane == 31)
        s_wsum[warp] = incl;
    __syncthreads();
    {
        const int ws = s_wsum[lane];
        int wi = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, wi, o);
            if (lane >= o)
                wi += t;
        }
        incl += __shfl_sync(FULL, wi - ws, warp);   /* block-inclusive */
        if (tid == CP_THREADS - 1)
            s_tstart[nt] = incl;
    }
    const int base = incl - cnt;   /* rank of this row's first point */
    if (owner && (tid & 31) == 0)
        s_tstart[tid >> 5] = base;
    __syncthreads();
    if (owner)
        s_rowrel[tid] = (unsigned short)(base - s_tstart[tid >> 5]);
    /* tile offsets within the CTA (float2 output pads odd tiles); the CTA's
     * count is published, then one grid barrier (an arrival counter on the
     * ticket word, bounded spin) and one read of the predecessors' counts */
    const int pad = a.pts_f2 ? 1 : 0;
    if (warp == 0) {
        int cq = 0;
        if (lane < nt)
            cq = s_tstart[lane + 1] - s_tstart[lane];
        const int pq = cq + (cq & pad);
        int ti = pq;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, ti, o);
            if (lane >= o)
                ti += t;
        }
        if (lane < nt)
            s_tbase[lane] = ti - pq;
        const int total = __shfl_sync(FULL, ti, 31);
        if (lane == 0) {
            s_total = total;
            lb_store(&a.tile_state[c], lb_pack(a.epoch, LB_AGG, (unsigned)total));
            __threadfence();
            atomicAdd(a.ticket, 1u);
            const unsigned target = a.ticket_base + (unsigned)nct;
            int spins = 0;
            while ((int)(*(volatile unsigned *)a.ticket - target) < 0) {
                if (++spins > LB_SPIN_LIMIT) {
                    atomicOr(a.status, HL_ST_LOOKBACK_TIMEOUT);
                    break;
                }
                __nanosleep(32);
            }
            __threadfence();
        }
    }
    __syncthreads();
    {
        int sum = 0;
        for (int j = tid; j < c; j += CP_THREADS)
            sum += (int)(unsigned)(lb_load(&a.tile_state[j]) & 0xffffffffu);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            sum += __shfl_xor_sync(FULL, sum, o);
        if (lane == 0)
            s_red[warp] = sum;
        __syncthreads();
        if (tid == 0) {
            int t = 0;
            for (int w = 0; w < CP_THREADS / 32; w++)
                t += s_red[w];
            s_excl = t;
        }
        __syncthreads();
    }
    const int excl = s_excl;
    if (tid < nt)
        a.tile_off[R.t0 + tid] = excl + s_tbase[tid];
    if (c == nct - 1 && tid == 0) {
        a.tile_off[a.ntiles] = excl + s_total;
        *a.count = excl + s_total;
    }
    /* scatter, one 16-pixel chunk per thread and round (chunk u = tid +
     * 1024 k): its rank is its row's start plus the points of the row's
     * chunks before it */
#pragma unroll
    for (int k = 0; k < CP_K; k++) {
        const int u = tid + k * CP_THREADS;
        if (u >= nu)
            break;
        uint32_t mm = s_mask[u];
        if (!mm)
            continue;
        const int row = u >> 3, ch = u & 7, tl = u >> 8;
        const uint4 q = reinterpret_cast<const uint4 *>(s_mask)[row];
        const unsigned long long lo = (unsigned long long)q.x | ((unsigned long long)q.y << 32);
        const unsigned long long hi = (unsigned long long)q.z | ((unsigned long long)q.w << 32);
        const int nb = 16 * ch;
        const int before = nb >= 64 ? __popcll(lo) + __popcll(hi & ((1ull << (nb - 64)) - 1ull))
                                    : __popcll(lo & ((1ull << nb) - 1ull));
        int pos = excl + s_tbase[tl] + s_rowrel[row] + before;
        const int x = s_x0[tl] + 16 * ch;
        const int y = s_y0[tl] + (row & 31);
        while (mm) {
            const int bb = __ffs(mm) - 1;
            mm &= mm - 1;
            if (a.pts_f2)
                a.pts_f2[pos] = make_float2((float)(x + bb), (float)y);
            else
                a.pts[pos] = (uint32_t)(x + bb) | ((uint32_t)y << 16);
            pos++;
        }
    }
    /* the sentinel (1e30, 0) of an odd float2 tile never votes inside an
     * accumulator (see hl_compact_kernel) */
    if (pad && tid < nt) {
        const int cq = s_tstart[tid + 1] - s_tstart[tid];
        if (cq & 1)
            a.pts_f2[excl + s_tbase[tid] + cq] = make_float2(1.0e30f, 0.0f);
    }
}

/* CTAs of the single-image compaction: about one per SM, at most CP_MAXT
 * tiles each; 0 when that needs more CTAs than can be resident at once
 * (callers then use hl_launch_compact) */
int hl_compact_persist_ctas(int ntiles, int sms)
{
    const int need = (ntiles + CP_MAXT - 1) / CP_MAXT;
    const int nct = std::max(1, std::min(ntiles, std::max(sms, need)));
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hl_compact_persist_kernel,
                                                      CP_THREADS, 0) != cudaSuccess)
        return 0;
    return nct <= per_sm * sms ? nct : 0;
}

cudaError_t hl_launch_compact_persist(const hl_compact_args *a, int nct, cudaStream_t s)
{
    return hl_launch_pdl(hl_compact_persist_kernel, dim3(nct), dim3(CP_THREADS), 0, s, true,
                         *a, nct);
}

cudaError_t hl_launch_compact(const hl_compact_args *a, cudaStream_t s)
{
    const int ngroups = a->imgs ? a->ngroups : (a->ntiles + CT_GROUP - 1) / CT_GROUP;
    return hl_launch_pdl(hl_compact_kernel, dim3(ngroups), dim3(HL_COMPACT_THREADS), 0, s,
                         false, *a);
}

/* Bounding box of an interleaved (x, y) list: bbox = {xmin, ymin, xmax, ymax}
 * (the reference's _findMinMaxCoordinates, okano_3_0/HoughLine.cu:287-334,
 * done on the device).  bbox must be preset to {INT_MAX, INT_MAX, INT_MIN,
 * INT_MIN}. */
__global__ void hl_bbox_kernel(const int *xy, int n, int *bbox)
{
    int xmin = 0x7fffffff, ymin = 0x7fffffff, xmax = (int)0x80000000,
        ymax = (int)0x80000000;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        int2 p = reinterpret_cast<const int2 *>(xy)[i];
        xmin = min(xmin, p.x);
        xmax = max(xmax, p.x);
        ymin = min(ymin, p.y);
        ymax = max(ymax, p.y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        xmin = min(xmin, __shfl_xor_sync(FULL, xmin, o));
        xmax = max(xmax, __shfl_xor_sync(FULL, xmax, o));
        ymin = min(ymin, __shfl_xor_sync(FULL, ymin, o));
        ymax = max(ymax, __shfl_xor_sync(FULL, ymax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&bbox[0], xmin);
        atomicMin(&bbox[1], ymin);
        atomicMax(&bbox[2], xmax);
        atomicMax(&bbox[3], ymax);
    }
}

cudaError_t hl_launch_bbox(const int *xy, int n, int *bbox, cudaStream_t s)
{
    int blocks = (n + 255) / 256;
    if (blocks > 1216)
        blocks = 1216;
    if (blocks < 1)
        blocks = 1;
    hl_bbox_kernel<<<blocks, 256, 0, s>>>(xy, n, bbox);
    return cudaGetLastError();
}
