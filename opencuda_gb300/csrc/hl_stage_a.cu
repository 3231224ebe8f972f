/*
 * hl_stage_a.cu -- cos/sin table and stage (a): edge-pixel compaction.
 *
 * Compaction replaces the flag / ScanArray / scatter chain of
 * ImgConvert::imgConvertToCst (okano_3_0/ImgConvert.cu:142-353,
 * okano_3_0/ScanArray.cu:1351+) with ONE pass: every CTA reads one
 * 128 x 32 tile with 16-byte vector loads, counts its 255-pixels, obtains the
 * tile's exclusive prefix by decoupled look-back over its predecessors'
 * published aggregates, and scatters packed coordinates.  The predicate is
 * the vote kernel's `pixel == 255` (okano_3_0/HoughLine.cu:125), not
 * ImgConvert's `>= 128`.
 *
 * HBM-bound: each image byte is read once (w*h bytes) and each edge point is
 * written once (4 bytes).
 */
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

__global__ void __launch_bounds__(HL_COMPACT_THREADS)
hl_compact_kernel(hl_compact_args a)
{
    __shared__ int s_tile;
    __shared__ int s_wsum[HL_COMPACT_THREADS / 32];
    __shared__ int s_base;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    /* Tiles are taken in ticket order, so every predecessor of a tile is
     * already resident when the tile looks back: the waits always end. */
    if (tid == 0)
        s_tile = (int)(atomicAdd(a.ticket, 1u) - a.ticket_base);
    __syncthreads();
    const int tile = s_tile;
    if (tile < 0 || tile >= a.ntiles)
        return;
    const int tx = tile % a.tiles_x, ty = tile / a.tiles_x;
    const int r = tid >> 3, ch = tid & 7;
    const int y = ty * HL_TILE_H + r;
    const int x0 = tx * HL_TILE_W + ch * 16;

    uint32_t m = 0;
    if (y < a.roi.h && x0 < a.roi.w) {
        const uint8_t *p = a.roi.base + (size_t)y * (size_t)a.roi.pitch + x0;
        if (x0 + 16 <= a.roi.w && (((uintptr_t)p) & 15u) == 0) {
            uint4 v = __ldcs((const uint4 *)p);
            m = eq255x4(v.x) | (eq255x4(v.y) << 4) | (eq255x4(v.z) << 8) |
                (eq255x4(v.w) << 12);
        } else {
            int lim = min(16, a.roi.w - x0);
            for (int i = 0; i < lim; i++)
                m |= (uint32_t)(p[i] == 255) << i;
        }
    }
    const int cnt = __popc(m);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o)
            incl += v;
    }
    if (lane == 31)
        s_wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int nw = HL_COMPACT_THREADS / 32;
        int ws = lane < nw ? s_wsum[lane] : 0;
        int wi = ws;
#pragma unroll
        for (int o = 1; o < nw; o <<= 1) {
            int v = __shfl_up_sync(FULL, wi, o);
            if (lane >= o)
                wi += v;
        }
        const int total = __shfl_sync(FULL, wi, nw - 1);
        if (lane < nw)
            s_wsum[lane] = wi - ws;
        const int excl = lookback(a.tile_state, tile, total, a.epoch, a.status);
        if (lane == 0) {
            s_base = excl;
            a.tile_off[tile] = excl;
            if (tile == a.ntiles - 1) {
                a.tile_off[a.ntiles] = excl + total;
                *a.count = excl + total;
            }
        }
    }
    __syncthreads();
    int pos = s_base + s_wsum[warp] + incl - cnt;
    const uint32_t yy = (uint32_t)y << 16;
    while (m) {
        int b = __ffs(m) - 1;
        m &= m - 1;
        a.pts[pos++] = (uint32_t)(x0 + b) | yy;
    }
}

cudaError_t hl_launch_compact(const hl_compact_args *a, cudaStream_t s)
{
    hl_compact_kernel<<<a->ntiles, HL_COMPACT_THREADS, 0, s>>>(*a);
    return cudaGetLastError();
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
