/*
 * hl_cnn.cu -- the proposal network's kernels: 3x3 convolutions as implicit
 * GEMMs on the 5th-generation tensor cores (tcgen05.mma, BF16 operands in
 * shared memory, FP32 accumulators in tensor memory), their backward passes,
 * the occupancy pooling and the fixed coarse Hough head.
 *
 * The reference has no learned component; this is the proposal stage of the
 * plain method's accelerated variant: a small CNN reads an average-pooled
 * edge map and predicts which coarse (theta, rho) cells hold lines, and the
 * exact int32 vote then runs only in those cells (hl_proposal.cpp).
 *
 * Activations are NHWC bfloat16 with C = 32 (64 bytes per pixel), the input
 * map is NHWC with C = 1.  Weights are [Cout][K] bfloat16 with K = tap * Cin
 * + ci (tap = ky * 3 + kx), K-major, so that one GEMM row of the weight
 * operand is one output channel.
 *
 * Implicit GEMM, one CTA of 128 threads per 128-pixel output tile:
 *   D[128 x N] = A[128 x K] * B[N x K]^T,
 *   A[m][k] = input pixel of output pixel m at tap k / Cin, channel k % Cin
 *   (zero outside the image), gathered into shared memory in the no-swizzle
 *   K-major core-matrix layout (8 rows x 16 bytes per core matrix), B the
 *   weights in the same layout.  Thread 0 issues K / 16 tcgen05.mma
 *   (M = 128, N = 32 or 16, K = 16) into a 32-column TMEM accumulator and
 *   commits them to an mbarrier; each warp then reads its 32 TMEM lanes
 *   (tcgen05.ld 32x32b) and runs the epilogue (bias, ReLU, bf16 store).
 */
#include "hl_internal.h"
#include "hl_cnn.h"

#include <cuda_bf16.h>

#define FULL 0xffffffffu
#define CNN_THREADS 128
#define CNN_TILE_M 128
#define CNN_WAIT_LIMIT (1 << 22)

/* ---- tcgen05 / mbarrier primitives ------------------------------------- */
__device__ __forceinline__ unsigned cnn_smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

/* Shared-memory matrix descriptor, no swizzle, K-major: start address,
 * leading-dimension byte offset (between the two 8-element K groups of one
 * MMA), stride byte offset (between 8-row groups), descriptor version 1. */
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr,
                                                        unsigned lbo,
                                                        unsigned sbo)
{
    unsigned long long d = 0;
    d |= (unsigned long long)((addr >> 4) & 0x3fffu);
    d |= (unsigned long long)((lbo >> 4) & 0x3fffu) << 16;
    d |= (unsigned long long)((sbo >> 4) & 0x3fffu) << 32;
    d |= 1ull << 46;   /* version */
    /* base offset 0, lbo mode 0, layout type 0 = no swizzle */
    return d;
}

/* Instruction descriptor of kind::f16: D f32, A and B bf16, both K-major,
 * no negation, N and M as given. */
__host__ __device__ constexpr unsigned mma_idesc(int M, int N)
{
    return (1u << 4)                       /* D format f32 */
           | (1u << 7)                     /* A format bf16 */
           | (1u << 10)                    /* B format bf16 */
           | ((unsigned)(N >> 3) << 17)    /* N / 8 */
           | ((unsigned)(M >> 4) << 24);   /* M / 16 */
}

__device__ __forceinline__ void cnn_mbar_init(unsigned long long *bar, unsigned n)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(cnn_smem_u32(bar)),
                 "r"(n)
                 : "memory");
}

__device__ __forceinline__ bool cnn_mbar_wait(unsigned long long *bar,
                                              unsigned parity)
{
    const unsigned a = cnn_smem_u32(bar);
    for (int i = 0; i < CNN_WAIT_LIMIT; i++) {
        unsigned ok;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], "
            "%2; selp.u32 %0, 1, 0, p; }"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok)
            return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_alloc32(unsigned *dst_smem)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;"
                 ::"r"(cnn_smem_u32(dst_smem))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc32(unsigned taddr)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(taddr)
                 : "memory");
}

__device__ __forceinline__ void umma_f16(unsigned tmem_d, unsigned long long adesc,
                                         unsigned long long bdesc, unsigned idesc,
                                         int accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(unsigned long long *bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
        ::"r"(cnn_smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

/* 32 consecutive fp32 columns of this thread's TMEM lane */
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&v)[32])
{
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
          "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
          "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
          "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
          "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++)
        v[i] = __uint_as_float(r[i]);
}

/* ---- the convolution ----------------------------------------------------- */

/* Shared memory of one CTA: A (128 rows x K) and B (N rows x K) in core
 * matrices.  Core matrix (row group g, K group q) of an operand with KG K
 * groups sits at ((g * KG) + q) * 128 bytes, so the two K groups of MMA step
 * s start at 2 s * 128 (LBO = 128) and consecutive row groups are KG * 128
 * apart (SBO). */
template <int KG, int NROWS>
struct ConvSmem {
    alignas(128) unsigned char a[CNN_TILE_M / 8][KG][128];
    alignas(128) unsigned char b[NROWS / 8][KG][128];
    unsigned long long bar;
    unsigned tmem;
    int tile;
};

/* Gather modes of the A operand. */
enum { GATHER_CONV = 0,        /* y[p] = sum w * x[p * stride - 1 + tap] */
       GATHER_CONVT2 = 1 };    /* x-gradient of a stride-2 conv:
                                  dx[p] = sum w * dy[(p + 1 - tap) / 2] */

/* One CTA per 128 output pixels, persistent over tiles.  Template:
 * CIN (1 or 32), N (GEMM N: 32, or 16 for a one-channel output padded with
 * zero weights), MODE (gather).  x: [B][H][W][CIN] bf16; y: [B][Ho][Wo][COUT]
 * bf16 (or f32 when y_f32 is set, COUT = 1). */
template <int CIN, int N, int MODE>
__global__ void __launch_bounds__(CNN_THREADS)
hl_conv3x3_kernel(hl_conv_args a)
{
    constexpr int K = (CIN == 1) ? 16 : 9 * CIN;   /* padded to 16 for CIN = 1 */
    constexpr int KG = K / 8;
    extern __shared__ __align__(128) unsigned char conv_raw[];
    ConvSmem<KG, N> &sm = *reinterpret_cast<ConvSmem<KG, N> *>(conv_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int HWo = a.Ho * a.Wo;
    const int ntiles = (a.B * HWo + CNN_TILE_M - 1) / CNN_TILE_M;

    /* weights -> B operand (once per CTA): row n = output channel, K group q
     * = 8 consecutive k; rows n >= cout are zero */
    for (int e = tid; e < N * KG; e += CNN_THREADS) {
        const int n = e / KG, q = e % KG;
        __nv_bfloat16 v8[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int k = q * 8 + j;
            const bool ok = n < a.cout && k < a.kreal;
            v8[j] = ok ? a.w[(size_t)n * a.kreal + k] : __float2bfloat16(0.0f);
        }
        unsigned char *dst = &sm.b[n >> 3][q][(n & 7) * 16];
        *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(v8);
    }
    if (warp == 0)
        tmem_alloc32(&sm.tmem);
    if (tid == 0) {
        cnn_mbar_init(&sm.bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    const unsigned tmem = sm.tmem;
    unsigned phase = 0;
    bool failed = false;

    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        /* A operand: row m = output pixel tile * 128 + m */
        if (CIN == 32) {
            /* thread m gathers row m (one output pixel): its coordinates once,
             * then one 16-byte cp.async per K group (tap q / 4, channels
             * (q % 4) * 8 .. +7) with compile-time tap offsets; every copy of
             * the tile in flight at once, zero-filled outside the image */
            static_assert(CNN_THREADS == CNN_TILE_M, "one thread per tile row");
            const int m = tid;
            const int p = tile * CNN_TILE_M + m;
            const bool row_ok = p < a.B * HWo;
            int bimg = 0, oy = 0, ox = 0;
            if (row_ok) {
                bimg = p / HWo;
                const int r = p - bimg * HWo;
                oy = r / a.Wo;
                ox = r - oy * a.Wo;
            }
            const __nv_bfloat16 *ximg = a.x + (size_t)bimg * a.H * a.W * 32;
            const unsigned arow = cnn_smem_u32(&sm.a[m >> 3][0][(m & 7) * 16]);
#pragma unroll
            for (int tap = 0; tap < 9; tap++) {
                const int ky = tap / 3, kx = tap % 3;
                int iy, ix;
                bool ok;
                if (MODE == GATHER_CONV) {
                    iy = oy * a.stride - 1 + ky;
                    ix = ox * a.stride - 1 + kx;
                    ok = row_ok && iy >= 0 && ix >= 0 && iy < a.H && ix < a.W;
                } else {
                    const int ty = oy + 1 - ky, tx = ox + 1 - kx;
                    iy = ty >> 1;
                    ix = tx >> 1;
                    ok = row_ok && ty >= 0 && tx >= 0 && !(ty & 1) && !(tx & 1) &&
                         iy < a.H && ix < a.W;
                }
                const __nv_bfloat16 *src = ok ? ximg + ((size_t)iy * a.W + ix) * 32 : a.x;
#pragma unroll
                for (int c = 0; c < 4; c++)
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;"
                                 ::"r"(arow + (unsigned)((tap * 4 + c) * 128)),
                                 "l"(src + c * 8), "r"(ok ? 16 : 0)
                                 : "memory");
            }
            asm volatile("cp.async.wait_all;" ::: "memory");
        } else {
            for (int e = tid; e < CNN_TILE_M * KG; e += CNN_THREADS) {
                const int m = e / KG, q = e % KG;
                const int p = tile * CNN_TILE_M + m;
                uint4 val = make_uint4(0u, 0u, 0u, 0u);
                if (p < a.B * HWo) {
                    const int bimg = p / HWo, r = p % HWo;
                    const int oy = r / a.Wo, ox = r % a.Wo;
                    /* CIN = 1: k = tap, 9 taps then zeros */
                    __nv_bfloat16 v8[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const int tap = q * 8 + j;
                        __nv_bfloat16 v = __float2bfloat16(0.0f);
                        if (tap < 9) {
                            const int ky = tap / 3, kx = tap % 3;
                            const int iy = oy * a.stride - 1 + ky;
                            const int ix = ox * a.stride - 1 + kx;
                            if (iy >= 0 && ix >= 0 && iy < a.H && ix < a.W)
                                v = a.x[((size_t)bimg * a.H + iy) * a.W + ix];
                        }
                        v8[j] = v;
                    }
                    val = *reinterpret_cast<const uint4 *>(v8);
                }
                *reinterpret_cast<uint4 *>(&sm.a[m >> 3][q][(m & 7) * 16]) = val;
            }
        }
        /* make the generic-proxy writes visible to the tensor cores */
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            tmem_fence_after();
            const unsigned abase = cnn_smem_u32(&sm.a[0][0][0]);
            const unsigned bbase = cnn_smem_u32(&sm.b[0][0][0]);
            constexpr unsigned idesc = mma_idesc(CNN_TILE_M, N);
#pragma unroll
            for (int s = 0; s < K / 16; s++) {
                const unsigned long long ad = smem_desc(abase + s * 256, 128, KG * 128);
                const unsigned long long bd = smem_desc(bbase + s * 256, 128, KG * 128);
                umma_f16(tmem, ad, bd, idesc, s > 0);
            }
            umma_commit(&sm.bar);
        }
        __syncwarp();
        const bool got = cnn_mbar_wait(&sm.bar, phase);
        phase ^= 1u;
        tmem_fence_after();
        if (!got) {
            failed = true;
            if (lane == 0)
                atomicOr(a.status, HL_ST_CNN_TIMEOUT);
        } else {
            /* epilogue: warp w holds rows 32 w .. 32 w + 31 (its TMEM lanes) */
            float v[32];
            tmem_ld32(tmem + ((unsigned)(32 * warp) << 16), v);
            const int m = 32 * warp + lane;
            const int p = tile * CNN_TILE_M + m;
            if (p < a.B * HWo) {
                if (a.y_f32) {
                    float o = v[0] + (a.bias ? a.bias[0] : 0.0f);
                    if (a.relu)
                        o = fmaxf(o, 0.0f);
                    a.y_f32[p] = o;
                } else {
                    __nv_bfloat16 o8[32];
#pragma unroll
                    for (int c = 0; c < 32; c++) {
                        float o = v[c] + ((a.bias && c < a.cout) ? a.bias[c] : 0.0f);
                        if (a.relu)
                            o = fmaxf(o, 0.0f);
                        if (c >= a.cout)
                            o = 0.0f;
                        o8[c] = __float2bfloat16(o);
                    }
                    uint4 *dst = reinterpret_cast<uint4 *>(a.y + (size_t)p * 32);
#pragma unroll
                    for (int c = 0; c < 4; c++)
                        dst[c] = reinterpret_cast<const uint4 *>(o8)[c];
                }
            }
        }
        /* TMEM reads and shared-memory reads done before the next tile */
        tmem_fence_before();
        __syncthreads();
        tmem_fence_after();
    }
    if (failed) {
        /* a commit that never arrived: nothing more is issued; wait once
         * more (bounded) so no MMA still writes the TMEM being released */
        cnn_mbar_wait(&sm.bar, phase);
    }
    __syncthreads();
    if (warp == 0)
        tmem_dealloc32(tmem);
}

template <int CIN, int N, int MODE>
static cudaError_t launch_conv(const hl_conv_args *a, int sms, cudaStream_t s)
{
    constexpr int K = (CIN == 1) ? 16 : 9 * CIN;
    const size_t smem = sizeof(ConvSmem<K / 8, N>) + 128;
    cudaError_t e = cudaFuncSetAttribute(hl_conv3x3_kernel<CIN, N, MODE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    const int ntiles = (a->B * a->Ho * a->Wo + CNN_TILE_M - 1) / CNN_TILE_M;
    /* CTAs per SM: 32-channel inputs hold ~92 KB of operands (two fit);
     * one-channel inputs ~5 KB (eight fit, 8 x 32 TMEM columns) */
    const int grid = std::max(1, std::min(ntiles, sms * (CIN == 1 ? 8 : 2)));
    hl_conv3x3_kernel<CIN, N, MODE><<<grid, CNN_THREADS, smem, s>>>(*a);
    return cudaGetLastError();
}

cudaError_t hl_launch_conv3x3(const hl_conv_args *a, int mode, cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (a->cin == 1 && a->cout <= 32 && mode == GATHER_CONV)
        return launch_conv<1, 32, GATHER_CONV>(a, sms, s);
    if (a->cin == 32 && a->cout <= 16 && mode == GATHER_CONV)
        return launch_conv<32, 16, GATHER_CONV>(a, sms, s);
    if (a->cin == 32 && a->cout <= 32 && mode == GATHER_CONV)
        return launch_conv<32, 32, GATHER_CONV>(a, sms, s);
    if (a->cin == 32 && a->cout <= 32 && mode == GATHER_CONVT2)
        return launch_conv<32, 32, GATHER_CONVT2>(a, sms, s);
    return cudaErrorInvalidValue;
}

/* ---- occupancy pooling ---------------------------------------------------- */

/* out[b][i][j] (side x side, bf16) = fraction of 255-pixels in the f x f
 * block (i * f.., j * f..) of image b's ROI; blocks past the ROI count as
 * empty.  One thread per output cell. */
__global__ void hl_pool_kernel(const hl_pool_img *imgs, int nimg, int side,
                               __nv_bfloat16 *out)
{
    const int per = side * side;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
         e < (size_t)nimg * per; e += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(e / per), r = (int)(e % per);
        const int i = r / side, j = r % side;
        const hl_pool_img im = imgs[b];
        const int f = im.factor;
        int cnt = 0;
        const int y0 = i * f, x0 = j * f;
        const int x1 = min(x0 + f, im.w);
        for (int y = y0; y < min(y0 + f, im.h); y++) {
            const uint8_t *row = im.base + (size_t)y * im.pitch;
            int x = x0;
            /* four bytes a load where the row allows it (255-bytes counted
             * with one byte-wise compare), the rest byte by byte */
            if ((((uintptr_t)(row + x)) & 3u) == 0)
                for (; x + 4 <= x1; x += 4)
                    cnt += __popc(__vcmpeq4(*reinterpret_cast<const unsigned *>(row + x),
                                            0xffffffffu)) >> 3;
            for (; x < x1; x++)
                cnt += row[x] == 255;
        }
        out[e] = __float2bfloat16((float)cnt / (float)(f * f));
    }
}

cudaError_t hl_launch_pool(const hl_pool_img *imgs, int nimg, int side,
                           __nv_bfloat16 *out, cudaStream_t s)
{
    const size_t n = (size_t)nimg * side * side;
    const int blocks = (int)std::min((n + 255) / 256, (size_t)4096);
    hl_pool_kernel<<<std::max(blocks, 1), 256, 0, s>>>(imgs, nimg, side, out);
    return cudaGetLastError();
}

/* ---- weight and bias gradients (CUDA cores, FP32) ------------------------ */

/* dw[co][tap * cin + ci] += sum over pixels of dy[p][co] * x[in(p, tap)][ci].
 * Thread (tap, ci) keeps 32 accumulators (one per co); a CTA walks chunks of
 * DW_CHUNK output pixels grid-stride, with the chunk's dy rows in shared
 * memory, and adds its sums into dw once at the end.  dy: [P][32] f32 (the
 * output gradient after the ReLU mask), x: bf16 NHWC with cin channels
 * (32-channel rows for cin = 32, one value for cin = 1). */
#define DW_CHUNK 64
__global__ void __launch_bounds__(288)
hl_conv_dw_kernel(hl_dw_args a)
{
    __shared__ float s_dy[DW_CHUNK][32];
    const int t = threadIdx.x;
    const int tap = t / 32 < 9 ? t / 32 : 8, ci = t % 32;
    const bool act = t < 9 * a.cin;   /* cin = 1: threads 0..8 (ci = t) */
    const int my_tap = a.cin == 32 ? tap : t, my_ci = a.cin == 32 ? ci : 0;
    const int ky = my_tap / 3, kx = my_tap % 3;
    float acc[32];
#pragma unroll
    for (int c = 0; c < 32; c++)
        acc[c] = 0.0f;
    const int HWo = a.Ho * a.Wo;
    const long long P = (long long)a.B * HWo;
    for (long long p0 = (long long)blockIdx.x * DW_CHUNK; p0 < P;
         p0 += (long long)gridDim.x * DW_CHUNK) {
        for (int e = t; e < DW_CHUNK * 32; e += blockDim.x) {
            const long long p = p0 + e / 32;
            s_dy[e / 32][e % 32] =
                (p < P && (e % 32) < a.dy_c) ? a.dy[p * a.dy_c + (e % 32)] : 0.0f;
        }
        __syncthreads();
        if (act) {
            for (int q = 0; q < DW_CHUNK; q++) {
                const long long p = p0 + q;
                if (p >= P)
                    break;
                const int b = (int)(p / HWo), r = (int)(p % HWo);
                const int oy = r / a.Wo, ox = r % a.Wo;
                const int iy = oy * a.stride - 1 + ky, ix = ox * a.stride - 1 + kx;
                float xv = 0.0f;
                if (iy >= 0 && ix >= 0 && iy < a.H && ix < a.W)
                    xv = __bfloat162float(
                        a.x[(((size_t)b * a.H + iy) * a.W + ix) * a.cin + my_ci]);
#pragma unroll
                for (int c = 0; c < 32; c++)
                    acc[c] = fmaf(s_dy[q][c], xv, acc[c]);
            }
        }
        __syncthreads();
    }
    if (act) {
        const int kreal = 9 * a.cin;
        const int k = my_tap * a.cin + my_ci;
        for (int c = 0; c < a.cout; c++)
            atomicAdd(&a.dw[(size_t)c * kreal + k], acc[c]);
    }
}

/* db[c] += sum over pixels of dy[p][c] (dy rows of dy_c values) */
__global__ void hl_bias_grad_kernel(const float *dy, int dy_c, long long P, int cout,
                                    float *db)
{
    __shared__ float s[32][33];
    const int c = threadIdx.x & 31, row = threadIdx.x >> 5;   /* 256 threads */
    float acc = 0.0f;
    if (c < dy_c)
        for (long long p = (long long)blockIdx.x * 8 + row; p < P;
             p += (long long)gridDim.x * 8)
            acc += dy[p * dy_c + c];
    s[row][c] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        float t = 0.0f;
        for (int r = 0; r < 8; r++)
            t += s[r][threadIdx.x];
        if (threadIdx.x < cout)
            atomicAdd(&db[threadIdx.x], t);
    }
}

cudaError_t hl_launch_conv_dw(const hl_dw_args *a, cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long P = (long long)a->B * a->Ho * a->Wo;
    const int chunks = (int)((P + DW_CHUNK - 1) / DW_CHUNK);
    hl_conv_dw_kernel<<<std::max(1, std::min(chunks, sms * 4)), 288, 0, s>>>(*a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !a->db)
        return e;
    const int blocks = (int)std::max(1LL, std::min((P + 7) / 8, (long long)sms * 4));
    hl_bias_grad_kernel<<<blocks, 256, 0, s>>>(a->dy, a->dy_c, P, a->cout, a->db);
    return cudaGetLastError();
}

/* dy (bf16 NHWC 32) * [y > 0] -> f32 [P][32] and a bf16 copy (the next
 * backward convolution's operand); y is the layer's ReLU output.  For a
 * one-channel gradient (dy32 == NULL): g [P] f32 -> bf16 [P]. */
__global__ void hl_relu_mask_kernel(const __nv_bfloat16 *dx, const __nv_bfloat16 *y,
                                    long long n, float *out_f32,
                                    __nv_bfloat16 *out_bf16)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        float g = __bfloat162float(dx[e]);
        if (y && !(__bfloat162float(y[e]) > 0.0f))
            g = 0.0f;
        if (out_f32)
            out_f32[e] = g;
        if (out_bf16)
            out_bf16[e] = __float2bfloat16(g);
    }
}

cudaError_t hl_launch_relu_mask(const __nv_bfloat16 *dx, const __nv_bfloat16 *y,
                                long long n, float *out_f32,
                                __nv_bfloat16 *out_bf16, cudaStream_t s)
{
    const int blocks = (int)std::max(1LL, std::min((n + 255) / 256, 8192LL));
    hl_relu_mask_kernel<<<blocks, 256, 0, s>>>(dx, y, n, out_f32, out_bf16);
    return cudaGetLastError();
}

/* ---- coarse Hough head ------------------------------------------------------ */

/* cos and sin of the coarse angles (t + 0.5) * pi / HL_HEAD_T, evaluated in
 * double on the host and rounded to float; passed by value */
struct HeadTrig {
    float c[HL_HEAD_T], s[HL_HEAD_T];
};

static const HeadTrig &head_trig()
{
    static HeadTrig t;
    static bool init = false;
    if (!init) {
        for (int i = 0; i < HL_HEAD_T; i++) {
            const double th = ((double)i + 0.5) * 3.14159265358979323846 / HL_HEAD_T;
            t.c[i] = (float)cos(th);
            t.s[i] = (float)sin(th);
        }
        init = true;
    }
    return t;
}

/* bin of evidence cell (qy, qx) of image geometry g at coarse angle t; every
 * operation rounded as written so the CPU oracle reproduces it */
__device__ __forceinline__ int head_bin(const hl_head_geom &g, int qy, int qx,
                                        float c, float s)
{
    const float x = __fmul_rn(__fadd_rn((float)qx, 0.5f), g.cell);
    const float y = __fmul_rn(__fadd_rn((float)qy, 0.5f), g.cell);
    const float rho = __fadd_rn(__fmul_rn(x, c), __fmul_rn(y, s));
    int r = (int)floorf(__fmul_rn(__fsub_rn(rho, g.rho_min), g.inv_rw));
    return min(max(r, 0), HL_HEAD_R - 1);
}

/* logits[b][t][r] = alpha * sum_{cells with bin r at angle t} e[b][cell] + beta
 * One CTA per (image, group of HEAD_TG angles), the group's [HEAD_TG][R] sums
 * in shared memory.  A thread walks one line of evidence cells for one angle
 * -- a column when the angle's rho changes less along y (|sin| < |cos|), else
 * a row -- keeping a running sum while consecutive cells fall in one bin and
 * adding it to that bin when the bin changes: the cells of a line mostly
 * share bins, so this issues a few shared reductions per line instead of one
 * per cell.  The sums are 64-bit fixed point (2^-24 units), so they do not
 * depend on the order of the additions. */
#define HEAD_TG 6
#define HEAD_FIX 16777216.0f
__global__ void __launch_bounds__(384)
hl_head_fwd_kernel(const float *e, int ev, const hl_head_geom *geo,
                   const float *ab, float *hsum, float *logits, HeadTrig tr)
{
    __shared__ unsigned long long sh[HEAD_TG * HL_HEAD_R];
    __shared__ float cs[HEAD_TG], sn[HEAD_TG];
    const int b = blockIdx.y, t0 = blockIdx.x * HEAD_TG;
    const int nt = min(HEAD_TG, HL_HEAD_T - t0);
    for (int i = threadIdx.x; i < HEAD_TG * HL_HEAD_R; i += blockDim.x)
        sh[i] = 0ull;
    if (threadIdx.x < nt) {
        cs[threadIdx.x] = tr.c[t0 + threadIdx.x];
        sn[threadIdx.x] = tr.s[t0 + threadIdx.x];
    }
    __syncthreads();
    const hl_head_geom g = geo[b];
    const float *eb = e + (size_t)b * ev * ev;
    for (int job = threadIdx.x; job < nt * ev; job += blockDim.x) {
        const int t = job / ev, line = job % ev;
        const float c = cs[t], sv = sn[t];
        const bool walk_y = fabsf(sv) < fabsf(c);
        unsigned long long run = 0ull;
        int cur = -1;
        for (int i = 0; i < ev; i++) {
            const int qy = walk_y ? i : line, qx = walk_y ? line : i;
            if (qy >= g.qh || qx >= g.qw)
                continue;
            const float v = eb[qy * ev + qx];
            if (v == 0.0f)
                continue;
            const int bin = head_bin(g, qy, qx, c, sv);
            if (bin != cur) {
                if (cur >= 0)
                    atomicAdd(&sh[t * HL_HEAD_R + cur], run);
                cur = bin;
                run = 0ull;
            }
            run += (unsigned long long)__float2ll_rn(v * HEAD_FIX);
        }
        if (cur >= 0)
            atomicAdd(&sh[t * HL_HEAD_R + cur], run);
    }
    __syncthreads();
    const float alpha = ab[0], beta = ab[1];
    for (int i = threadIdx.x; i < nt * HL_HEAD_R; i += blockDim.x) {
        const size_t o = (size_t)b * HL_HEAD_T * HL_HEAD_R + (size_t)t0 * HL_HEAD_R + i;
        const float sum = (float)((double)(long long)sh[i] * (1.0 / HEAD_FIX));
        hsum[o] = sum;
        logits[o] = alpha * sum + beta;
    }
}

/* de[b][cell] = alpha * sum_t dz[b][t][bin(cell, t)] (the gather transpose of
 * the head); one CTA per (image, 512 cells), each thread one cell summing its
 * angles in order */
__global__ void __launch_bounds__(512)
hl_head_bwd_kernel(const float *dz, int ev, const hl_head_geom *geo,
                   const float *ab, float *de, HeadTrig tr)
{
    __shared__ float sd[HL_HEAD_T * HL_HEAD_R];
    __shared__ float cs[HL_HEAD_T], sn[HL_HEAD_T];
    const int b = blockIdx.y;
    for (int i = threadIdx.x; i < HL_HEAD_T * HL_HEAD_R; i += blockDim.x)
        sd[i] = dz[(size_t)b * HL_HEAD_T * HL_HEAD_R + i];
    if (threadIdx.x < HL_HEAD_T) {
        cs[threadIdx.x] = tr.c[threadIdx.x];
        sn[threadIdx.x] = tr.s[threadIdx.x];
    }
    __syncthreads();
    const hl_head_geom g = geo[b];
    const float alpha = ab[0];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ev * ev;
         p += gridDim.x * blockDim.x) {
        const int qy = p / ev, qx = p % ev;
        float acc = 0.0f;
        if (qy < g.qh && qx < g.qw)
            for (int t = 0; t < HL_HEAD_T; t++)
                acc += sd[t * HL_HEAD_R + head_bin(g, qy, qx, cs[t], sn[t])];
        de[(size_t)b * ev * ev + p] = alpha * acc;
    }
}

cudaError_t hl_launch_head_fwd(const float *e, int ev, const hl_head_geom *geo,
                               int nimg, const float *ab, float *hsum,
                               float *logits, cudaStream_t s)
{
    hl_head_fwd_kernel<<<dim3((HL_HEAD_T + HEAD_TG - 1) / HEAD_TG, nimg), 384, 0, s>>>(
        e, ev, geo, ab, hsum, logits, head_trig());
    return cudaGetLastError();
}

cudaError_t hl_launch_head_bwd(const float *dz, int ev, const hl_head_geom *geo,
                               int nimg, const float *ab, float *de, cudaStream_t s)
{
    hl_head_bwd_kernel<<<dim3((unsigned)((ev * ev + 511) / 512), nimg), 512, 0, s>>>(
        dz, ev, geo, ab, de, head_trig());
    return cudaGetLastError();
}

/* ---- loss ------------------------------------------------------------------- */

/* Weighted binary cross-entropy on logits: per cell
 * l = -(wpos * y * log s + (1 - y) * log(1 - s)), s = sigmoid(z); dz = dl/dz /
 * n; also d alpha = sum dz * hsum, d beta = sum dz and the summed loss. */
__global__ void hl_bce_kernel(const float *z, const float *y, const float *hsum,
                              long long n, float wpos, float *dz, float *dab,
                              float *loss)
{
    __shared__ float r[3][256];
    float la = 0.0f, ga = 0.0f, gb = 0.0f;
    const float inv = 1.0f / (float)n;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const float zz = z[e], yy = y[e];
        /* log(1 + exp(-|z|)) form, stable for large |z| */
        const float sp = log1pf(expf(-fabsf(zz)));
        const float log_s = fminf(zz, 0.0f) - sp;       /* log sigmoid(z) */
        const float log_1s = fminf(-zz, 0.0f) - sp;     /* log(1 - sigmoid(z)) */
        la += -(wpos * yy * log_s + (1.0f - yy) * log_1s);
        const float sg = 1.0f / (1.0f + expf(-zz));
        const float g = (wpos * yy * (sg - 1.0f) + (1.0f - yy) * sg) * inv;
        dz[e] = g;
        ga += g * hsum[e];
        gb += g;
    }
    r[0][threadIdx.x] = la;
    r[1][threadIdx.x] = ga;
    r[2][threadIdx.x] = gb;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int k = 0; k < 3; k++)
                r[k][threadIdx.x] += r[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(loss, r[0][0] * inv);
        atomicAdd(&dab[0], r[1][0]);
        atomicAdd(&dab[1], r[2][0]);
    }
}

cudaError_t hl_launch_bce(const float *z, const float *y, const float *hsum,
                          long long n, float wpos, float *dz, float *dab,
                          float *loss, cudaStream_t s)
{
    hl_bce_kernel<<<256, 256, 0, s>>>(z, y, hsum, n, wpos, dz, dab, loss);
    return cudaGetLastError();
}

/* ---- Adam and weight layouts ---------------------------------------------- */

__global__ void hl_adam_kernel(float *w, const float *g, float *m, float *v, int n,
                               float lr, float b1, float b2, float eps, float c1,
                               float c2, float clip)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const float gi = fminf(fmaxf(g[i], -clip), clip);
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

cudaError_t hl_launch_adam(float *w, const float *g, float *m, float *v, int n,
                           float lr, int step, float clip, cudaStream_t s)
{
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f / (1.0f - powf(b1, (float)step));
    const float c2 = 1.0f / (1.0f - powf(b2, (float)step));
    hl_adam_kernel<<<(n + 255) / 256, 256, 0, s>>>(w, g, m, v, n, lr, b1, b2, 1e-8f,
                                                   c1, c2, clip);
    return cudaGetLastError();
}

/* FP32 master weights [cout][9 * cin] -> the bf16 operand of one layer:
 * mode 0 forward (same layout), mode 1 flipped and transposed ([cin][tap][cout]
 * with tap -> 8 - tap: the stride-1 input gradient as a convolution), mode 2
 * transposed ([cin][tap][cout]: the stride-2 input-gradient gather). */
__global__ void hl_weight_layout_kernel(const float *w, int cout, int cin, int mode,
                                        __nv_bfloat16 *out)
{
    const int n = cout * 9 * cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const int co = i / (9 * cin), r = i % (9 * cin);
        const int tap = r / cin, ci = r % cin;
        const float v = w[i];
        if (mode == 0)
            out[i] = __float2bfloat16(v);
        else if (mode == 1)
            out[((size_t)ci * 9 + (8 - tap)) * cout + co] = __float2bfloat16(v);
        else
            out[((size_t)ci * 9 + tap) * cout + co] = __float2bfloat16(v);
    }
}

cudaError_t hl_launch_weight_layout(const float *w, int cout, int cin, int mode,
                                    __nv_bfloat16 *out, cudaStream_t s)
{
    const int n = cout * 9 * cin;
    hl_weight_layout_kernel<<<(n + 255) / 256, 256, 0, s>>>(w, cout, cin, mode, out);
    return cudaGetLastError();
}

__global__ void hl_f32_to_bf16_kernel(const float *in, long long n, __nv_bfloat16 *out)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x)
        out[e] = __float2bfloat16(in[e]);
}

cudaError_t hl_launch_f32_to_bf16(const float *in, long long n, __nv_bfloat16 *out,
                                  cudaStream_t s)
{
    const int blocks = (int)std::max(1LL, std::min((n + 255) / 256, 8192LL));
    hl_f32_to_bf16_kernel<<<blocks, 256, 0, s>>>(in, n, out);
    return cudaGetLastError();
}
