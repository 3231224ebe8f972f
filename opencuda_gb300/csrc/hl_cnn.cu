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
        for (int e = tid; e < CNN_TILE_M * KG; e += CNN_THREADS) {
            const int m = e / KG, q = e % KG;
            const int p = tile * CNN_TILE_M + m;
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (p < a.B * HWo) {
                const int bimg = p / HWo, r = p % HWo;
                const int oy = r / a.Wo, ox = r % a.Wo;
                if (CIN == 32) {
                    /* K group q = tap q / 4, channels (q % 4) * 8 .. +7 */
                    const int tap = q >> 2, c0 = (q & 3) * 8;
                    const int ky = tap / 3, kx = tap % 3;
                    int iy, ix;
                    bool ok;
                    if (MODE == GATHER_CONV) {
                        iy = oy * a.stride - 1 + ky;
                        ix = ox * a.stride - 1 + kx;
                        ok = iy >= 0 && ix >= 0 && iy < a.H && ix < a.W;
                    } else {
                        const int ty = oy + 1 - ky, tx = ox + 1 - kx;
                        iy = ty >> 1;
                        ix = tx >> 1;
                        ok = ty >= 0 && tx >= 0 && !(ty & 1) && !(tx & 1) &&
                             iy < a.H && ix < a.W;
                    }
                    if (ok)
                        val = *reinterpret_cast<const uint4 *>(
                            a.x + (((size_t)bimg * a.H + iy) * a.W + ix) * 32 + c0);
                } else {
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
            }
            *reinterpret_cast<uint4 *>(&sm.a[m >> 3][q][(m & 7) * 16]) = val;
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
    const int grid = std::max(1, std::min(ntiles, sms * 2));
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
