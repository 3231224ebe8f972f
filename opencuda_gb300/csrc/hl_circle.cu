/*
 * hl_circle.cu -- HoughCircle on the HoughLine engine (the image path of
 * HoughCircle::houghcircle, okano_3_0/HoughCircle.cu:927-1165): the edge
 * pixels come from the same compaction, votes go into a (radius, row,
 * column) accumulator, then a local-maximum pass and a one-CTA tail.
 *
 *   hl_circle_vote_kernel  -- every edge point votes, for every radius, the
 *       eight octant points of the reference's midpoint circle
 *       (okano_3_0/HoughCircle.cu:187-245: x = 0, y = r, d = 3 - 2r; while
 *       x < y ...; points on the axes twice).  The (radius, x, y) steps of
 *       every radius are tabulated once on the host; a CTA takes a point at a
 *       time and its threads the table entries, so a point's votes issue in
 *       parallel; each lands with red.global in the L2-resident accumulator.
 *   hl_circle_peaks_kernel -- okano_3_0/HoughCircle.cu:321-370: v above the
 *       threshold, above the left and upper neighbours and at least the right
 *       and lower ones (zero outside the ROI), per radius; the keys
 *       (votes << 32 | ~index) appended with one atomic per warp.
 *   hl_circle_final_kernel -- one CTA: rank sort (votes descending, index
 *       ascending: the deviation from the reference's shear sort is only the
 *       order of equal votes), decode (:632-657), the greedy merge of
 *       _recalCirParam (:809-871) on one warp, output with the ROI offset.
 */
#include "hl_internal.h"

#define FULL 0xffffffffu

/* ---- vote ---------------------------------------------------------------- */

/* tab[e] = {z, x | y << 16}: step (x, y) of radius rmin + z */
__global__ void __launch_bounds__(256)
hl_circle_vote_kernel(hl_circle_vote_args a)
{
    extern __shared__ int2 s_tab[];
    hl_pdl_begin();
    for (int e = threadIdx.x; e < a.ntab; e += blockDim.x)
        s_tab[e] = a.tab[e];
    __syncthreads();
    const int n = *a.count;
    const size_t plane = (size_t)a.w * a.h;
    for (int p = blockIdx.x; p < n; p += gridDim.x) {
        const float2 pt = a.pts[p];
        if (!(pt.x < 1.0e29f))
            continue;   /* the compaction's sentinel of an odd tile */
        const int x0 = (int)pt.x, y0 = (int)pt.y;
        for (int e = threadIdx.x; e < a.ntab; e += blockDim.x) {
            const int2 t = s_tab[e];
            const int ox = t.y & 0xffff, oy = t.y >> 16;
            int32_t *acc = a.acc + (size_t)t.x * plane;
            const int xs[8] = {x0 + ox, x0 + ox, x0 - ox, x0 - ox,
                               x0 + oy, x0 + oy, x0 - oy, x0 - oy};
            const int ys[8] = {y0 + oy, y0 - oy, y0 + oy, y0 - oy,
                               y0 + ox, y0 - ox, y0 + ox, y0 - ox};
#pragma unroll
            for (int q = 0; q < 8; q++)
                if (xs[q] >= 0 && xs[q] < a.w && ys[q] >= 0 && ys[q] < a.h)
                    atomicAdd(acc + (size_t)ys[q] * a.w + xs[q], 1);
        }
    }
}

/* ---- peaks --------------------------------------------------------------- */

__global__ void __launch_bounds__(256)
hl_circle_peaks_kernel(hl_circle_peak_args a)
{
    hl_pdl_begin();
    const long long total = (long long)a.nr * a.h * a.w;
    const int lane = threadIdx.x & 31;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < total;
         base += (long long)gridDim.x * blockDim.x) {
        const long long i = base + threadIdx.x;
        bool is = false;
        int v = 0;
        if (i < total) {
            const int x = (int)(i % a.w);
            const long long zy = i / a.w;
            const int y = (int)(zy % a.h);
            const int32_t *p = a.acc + i;
            v = p[0];
            if (v > a.threshold) {
                const int L = x > 0 ? p[-1] : 0;
                const int R = x + 1 < a.w ? p[1] : 0;
                const int U = y > 0 ? p[-a.w] : 0;
                const int D = y + 1 < a.h ? p[a.w] : 0;
                is = v > L && v >= R && v > U && v >= D;
            }
        }
        const unsigned b = __ballot_sync(FULL, is);
        if (!b)
            continue;
        int pos = 0;
        if (lane == 0)
            pos = atomicAdd(a.ncand, __popc(b));
        pos = __shfl_sync(FULL, pos, 0) + __popc(b & ((1u << lane) - 1u));
        if (is) {
            if (pos < a.cap)
                a.keys[pos] = ((unsigned long long)(unsigned)v << 32) |
                              (unsigned)(~(unsigned)i);
            else
                atomicOr(a.status, HL_ST_CAND_OVERFLOW);
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

cudaError_t hl_launch_circle_vote(const hl_circle_vote_args *a, int sms, cudaStream_t s)
{
    const size_t smem = sizeof(int2) * (size_t)a->ntab;
    cudaError_t e = cudaFuncSetAttribute(hl_circle_vote_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    return hl_launch_pdl(hl_circle_vote_kernel, dim3(sms * 8), dim3(256), smem, s, false, *a);
}

cudaError_t hl_launch_circle_peaks(const hl_circle_peak_args *a, int sms, cudaStream_t s)
{
    const long long total = (long long)a->nr * a->h * a->w;
    long long blocks = (total + 255) / 256;
    if (blocks > (long long)sms * 16)
        blocks = (long long)sms * 16;
    return hl_launch_pdl(hl_circle_peaks_kernel, dim3((unsigned)blocks), dim3(256), 0, s,
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
