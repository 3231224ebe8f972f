/*
 * hl_vote.cu -- stage (b): (theta, rho) int32 voting.
 *
 * Vote rule (okano_3_0/HoughLine.cu:86-130): an edge point (x, y) adds one
 * to bin (k, trunc(fl(x*cos_k) + fl(y*sin_k))) for every k.  The products and
 * the sum are rounded separately (__fmul_rn/__fadd_rn: no FMA contraction),
 * the float is truncated toward zero (the reference's +-0.5 step after the
 * (int) cast is a no-op), and cos_k/sin_k come from the GPU-evaluated table.
 *
 * Work decomposition.  A CTA owns a (theta slice, rho window) block of the
 * accumulator in shared memory: 32 thetas (one per lane) x win_rows rho bins,
 * laid out acc[row][lane].  A warp takes one point at a time; its 32 lanes
 * add to 32 different thetas of the same point, i.e. 32 different banks, so
 * every shared atomic instruction is conflict-free and no two lanes ever hit
 * one address (the aggregation a warp-aggregated atomic would buy is built
 * into the layout).  Points arrive tile-major from stage (a); a CTA whose
 * window does not cover the whole rho range skips tiles whose rho interval
 * over the slice misses its window.  Each CTA finally stores its block with
 * coalesced 128-byte rows into acc[R][Tp] -- every bin is written exactly
 * once, so the global accumulator needs no clearing.
 */
#include "hl_internal.h"

#define FULL 0xffffffffu
#define LIST_CAP 1024

template <bool UNIT>
__device__ __forceinline__ int rho_of(float x, float y, float c, float s,
                                      float irho)
{
    float a = __fmul_rn(x, c);
    float b = __fmul_rn(y, s);
    if (!UNIT) {
        a = __fmul_rn(a, irho);
        b = __fmul_rn(b, irho);
    }
    return __float2int_rz(__fadd_rn(a, b));
}

/* Conservative test: can any point of tile t vote into rho bins
 * [lo_bin, hi_bin] for a theta in [k0, k1]?  rho(x, y, th) is linear in
 * (x, y) for fixed th, so its extremes over the tile lie at the corners; over
 * th in [th0, th1] (within [0, pi)) a corner's value |p| cos(th - phi), phi in
 * [0, pi/2], has no interior minimum and an interior maximum |p| only when
 * phi lies between th0 and th1.  Two bins of slack cover float rounding. */
__device__ __forceinline__ bool tile_hits(int t, int tiles_x, int w, int h,
                                          float c0, float s0, float c1,
                                          float s1, float lo_bin,
                                          float hi_bin, float irho)
{
    int tx = t % tiles_x, ty = t / tiles_x;
    float xa = (float)(tx * HL_TILE_W);
    float xb = (float)min(tx * HL_TILE_W + HL_TILE_W - 1, w - 1);
    float ya = (float)(ty * HL_TILE_H);
    float yb = (float)min(ty * HL_TILE_H + HL_TILE_H - 1, h - 1);
    float mn = 3.0e38f, mx = -3.0e38f;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float x = (i & 1) ? xb : xa;
        float y = (i & 2) ? yb : ya;
        float f0 = x * c0 + y * s0;
        float f1 = x * c1 + y * s1;
        mn = fminf(mn, fminf(f0, f1));
        float hi = fmaxf(f0, f1);
        float tol = 1e-3f * (x + y) + 1e-3f;
        if (c0 * y - s0 * x >= -tol && x * s1 - y * c1 >= -tol)
            hi = fmaxf(hi, sqrtf(x * x + y * y) + 1.0f);
        mx = fmaxf(mx, hi);
    }
    mn = mn * irho - 3.0f;
    mx = mx * irho + 3.0f;
    return mn <= hi_bin && mx >= lo_bin;
}

template <bool UNIT>
__global__ void __launch_bounds__(1024, 1)
hl_vote_kernel(hl_vote_args a)
{
    extern __shared__ __align__(16) int s_acc[];   /* win_rows * 32 */
    __shared__ int s_list[LIST_CAP];
    __shared__ int s_nlist, s_next;

    const int tid = threadIdx.x, lane = tid & 31;
    const int slice = blockIdx.x, win = blockIdx.y;
    const int k0 = slice * HL_SLICE;
    const int k = k0 + lane;
    const bool kvalid = k < a.T;
    const float c = a.cosv[k], s = a.sinv[k];   /* table padded to Tp */
    const int w0 = win * a.win_rows;
    const int rows = min(a.win_rows, a.R - w0);
    const int row_base = a.rho_min + w0;        /* rho bin of local row 0 */

    for (int i = tid; i < rows * HL_SLICE; i += blockDim.x)
        s_acc[i] = 0;

    const int klast = min(k0 + HL_SLICE - 1, a.T - 1);
    const float c0 = a.cosv[k0], s0 = a.sinv[k0];
    const float c1 = a.cosv[klast], s1 = a.sinv[klast];
    const float lo_bin = (float)row_base, hi_bin = (float)(row_base + rows - 1);

    for (int t0 = 0; t0 < a.ntiles; t0 += LIST_CAP) {
        if (tid == 0) {
            s_nlist = 0;
            s_next = 0;
        }
        __syncthreads();
        const int t1 = min(a.ntiles, t0 + LIST_CAP);
        for (int t = t0 + tid; t < t1; t += blockDim.x) {
            if (a.tile_off[t + 1] == a.tile_off[t])
                continue;
            if (a.nwin == 1 ||
                tile_hits(t, a.tiles_x, a.w, a.h, c0, s0, c1, s1, lo_bin,
                          hi_bin, a.irho)) {
                int pos = atomicAdd(&s_nlist, 1);
                s_list[pos] = t;
            }
        }
        __syncthreads();
        const int nl = s_nlist;
        while (true) {
            int item = 0;
            if (lane == 0)
                item = atomicAdd(&s_next, 1);
            item = __shfl_sync(FULL, item, 0);
            if (item >= nl)
                break;
            const int t = s_list[item];
            const int beg = a.tile_off[t], end = a.tile_off[t + 1];
            for (int b = beg; b < end; b += 32) {
                const int i = b + lane;
                const uint32_t pk = (i < end) ? __ldg(&a.pts[i]) : 0u;
                const float xf = (float)(pk & 0xffffu);
                const float yf = (float)(pk >> 16);
                const int nb = min(32, end - b);
                for (int j = 0; j < nb; j++) {
                    const float x = __shfl_sync(FULL, xf, j);
                    const float y = __shfl_sync(FULL, yf, j);
                    const int row = rho_of<UNIT>(x, y, c, s, a.irho) - row_base;
                    if (kvalid && (unsigned)row < (unsigned)rows)
                        atomicAdd(&s_acc[row * HL_SLICE + lane], 1);
                }
            }
        }
        __syncthreads();
    }

    /* store the block: row r of the window -> acc[(w0 + r) * Tp + k0 ..] */
    int4 *dst4 = reinterpret_cast<int4 *>(a.acc);
    const int4 *src4 = reinterpret_cast<const int4 *>(s_acc);
    const int tp4 = a.Tp >> 2;
    for (int i = tid; i < rows * (HL_SLICE / 4); i += blockDim.x) {
        int r = i >> 3, q = i & 7;
        dst4[(size_t)(w0 + r) * tp4 + (k0 >> 2) + q] = src4[i];
    }
}

size_t hl_vote_smem_bytes(int win_rows)
{
    return (size_t)win_rows * HL_SLICE * sizeof(int);
}

cudaError_t hl_launch_vote(const hl_vote_args *a, int threads, cudaStream_t s)
{
    dim3 grid(a->Tp / HL_SLICE, a->nwin);
    size_t smem = hl_vote_smem_bytes(a->win_rows);
    cudaError_t e;
    if (a->irho == 1.0f) {
        e = cudaFuncSetAttribute(hl_vote_kernel<true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess)
            return e;
        hl_vote_kernel<true><<<grid, threads, smem, s>>>(*a);
    } else {
        e = cudaFuncSetAttribute(hl_vote_kernel<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess)
            return e;
        hl_vote_kernel<false><<<grid, threads, smem, s>>>(*a);
    }
    return cudaGetLastError();
}

/* Voting over an interleaved int (x, y) list (the guidingset path,
 * okano_3_0/HoughLine.cu:133-165).  No tile order here, so every window
 * reads every point; the per-vote row test keeps it exact. */
template <bool UNIT>
__global__ void __launch_bounds__(1024, 1)
hl_vote_points_kernel(const int2 *xy, int n, const float *cosv,
                      const float *sinv, int T, int Tp, int rho_min, int R,
                      int win_rows, float irho, int32_t *acc)
{
    extern __shared__ __align__(16) int s_acc[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    const int k0 = blockIdx.x * HL_SLICE, k = k0 + lane;
    const bool kvalid = k < T;
    const float c = cosv[k], s = sinv[k];
    const int w0 = blockIdx.y * win_rows;
    const int rows = min(win_rows, R - w0);
    const int row_base = rho_min + w0;
    for (int i = tid; i < rows * HL_SLICE; i += blockDim.x)
        s_acc[i] = 0;
    __syncthreads();
    for (int b = warp * 32; b < n; b += nwarps * 32) {
        const int i = b + lane;
        int2 p = (i < n) ? xy[i] : make_int2(0, 0);
        const float xf = (float)p.x, yf = (float)p.y;
        const int nb = min(32, n - b);
        for (int j = 0; j < nb; j++) {
            const float x = __shfl_sync(FULL, xf, j);
            const float y = __shfl_sync(FULL, yf, j);
            const int row = rho_of<UNIT>(x, y, c, s, irho) - row_base;
            if (kvalid && (unsigned)row < (unsigned)rows)
                atomicAdd(&s_acc[row * HL_SLICE + lane], 1);
        }
    }
    __syncthreads();
    int4 *dst4 = reinterpret_cast<int4 *>(acc);
    const int4 *src4 = reinterpret_cast<const int4 *>(s_acc);
    const int tp4 = Tp >> 2;
    for (int i = tid; i < rows * (HL_SLICE / 4); i += blockDim.x) {
        int r = i >> 3, q = i & 7;
        dst4[(size_t)(w0 + r) * tp4 + (k0 >> 2) + q] = src4[i];
    }
}

cudaError_t hl_launch_vote_points(const int *xy, int n, const float *cosv,
                                  const float *sinv, int T, int Tp,
                                  int rho_min, int R, int win_rows, int nwin,
                                  float irho, int32_t *acc, int threads,
                                  cudaStream_t s)
{
    dim3 grid(Tp / HL_SLICE, nwin);
    size_t smem = hl_vote_smem_bytes(win_rows);
    cudaError_t e;
    if (irho == 1.0f) {
        e = cudaFuncSetAttribute(hl_vote_points_kernel<true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess)
            return e;
        hl_vote_points_kernel<true><<<grid, threads, smem, s>>>(
            reinterpret_cast<const int2 *>(xy), n, cosv, sinv, T, Tp, rho_min,
            R, win_rows, irho, acc);
    } else {
        e = cudaFuncSetAttribute(hl_vote_points_kernel<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess)
            return e;
        hl_vote_points_kernel<false><<<grid, threads, smem, s>>>(
            reinterpret_cast<const int2 *>(xy), n, cosv, sinv, T, Tp, rho_min,
            R, win_rows, irho, acc);
    }
    return cudaGetLastError();
}

/* Shared-memory atomic ceiling: every lane adds to its own bank, 8
 * independent addresses per thread per iteration, 1024 threads per CTA, two
 * CTAs per SM.  The counters are summed into *sink so nothing is dead. */
__global__ void __launch_bounds__(1024, 2)
hl_atomic_bench_kernel(int iters, int *sink)
{
    __shared__ int s[8 * 1024];
    const int tid = threadIdx.x;
    for (int i = tid; i < 8 * 1024; i += blockDim.x)
        s[i] = 0;
    __syncthreads();
    const int lane = tid & 31, warp = tid >> 5;
    int *base = s + (warp & 31) * 256 + lane;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
            atomicAdd(base + u * 32, 1);
    }
    __syncthreads();
    if (tid == 0) {
        int acc = 0;
        for (int i = 0; i < 8 * 1024; i += 97)
            acc += s[i];
        atomicAdd(sink, acc);
    }
}

cudaError_t hl_launch_atomic_bench(int iters, int *sink, cudaStream_t s,
                                   int *blocks_out, int *threads_out)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int blocks = sms * 2;
    hl_atomic_bench_kernel<<<blocks, 1024, 0, s>>>(iters, sink);
    if (blocks_out)
        *blocks_out = blocks;
    if (threads_out)
        *threads_out = 1024;
    return cudaGetLastError();
}
