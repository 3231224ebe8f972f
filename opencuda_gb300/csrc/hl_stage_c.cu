/*
 * hl_stage_c.cu -- stage (c): peak NMS + threshold, then rank, decode, merge
 * and truncate, all on the device.
 *
 * The reference finds peaks with _findlocalMaxKer (okano_3_0/HoughLine.cu:
 * 168-213, racy and unchecked at its edges), copies two accumulator-sized
 * arrays to the host and ranks / merges there (:781-948).  Here:
 *   hl_peaks_kernel   -- bounds-checked peak rule, peaks appended as
 *                        64-bit keys (votes << 32 | ~index): over the bins
 *                        the vote noted above the threshold (batches), or one
 *                        read of acc[R][Tp] (one image; HBM / L2 bound);
 *   hl_finalize_kernel -- one CTA: top-M selection (MSD radix select when the
 *                        peaks exceed one 1024-key chunk), rank sort of the
 *                        chunk (keys are unique), the reference's float
 *                        decode, the pairwise predecessor bitmask, and the
 *                        greedy merge resolved by one warp word by word;
 *                        writes min(survivors, linesmax) LineParam records
 *                        (hl_finalize_cluster_kernel: the same for one image
 *                        with the sort and the bitmask spread over a
 *                        cluster).
 * Ranking is canonical: votes descending, then the reference raster index
 * (rho-major, theta-minor) ascending -- the reference's Shell sort
 * (:853-873) is unstable, so ties are ordered by index here.
 */
#include "hl_internal.h"
#include "hl_device.cuh"

#include <math.h>

#include <algorithm>

#include <cooperative_groups.h>
namespace cg = cooperative_groups;

#define FULL 0xffffffffu
#define FIN_THREADS 1024
#define FIN_CHUNK 1024
#define FIN_SCACHE 1024

/* The peak rule (okano_3_0/HoughLine.cu:195-199, bounds-checked: zero
 * outside the accumulator) for bin k of row `row` (p points at it), which
 * exceeds the threshold; a peak is appended as its key.  Scalar loads: the
 * bins are rare, and the kernel keeps few registers. */
__device__ __forceinline__ void peak_bin(const int32_t *p, unsigned long long *keys, int *ncand,
                                         int R, int cap, int T, int Tp, int row, int k,
                                         int *status)
{
    const int x = p[0];
    const int W = k > 0 ? p[-1] : 0;
    const int E = k + 1 < T ? p[1] : 0;
    const int N = row > 0 ? p[-Tp] : 0;
    const int S = row + 1 < R ? p[Tp] : 0;
    if (x > W && x >= E && x > N && x >= S) {
        const unsigned idx = (unsigned)row * (unsigned)T + (unsigned)k;
        const int pos = atomicAdd(ncand, 1);
        if (pos < cap)
            keys[pos] = ((unsigned long long)(unsigned)x << 32) | (unsigned)(~idx);
        else
            atomicOr(status, HL_ST_CAND_OVERFLOW);
    }
}

/* The peak rule for every bin above the threshold.  When the vote and the
 * merge noted all of them (the usual case: they are rare), each thread
 * takes noted bins and reads only their neighbours -- no accumulator is
 * read as a whole.  Otherwise one read of every accumulator at the memory
 * system's speed.  Work units are taken grid-stride: with several images (chunks != NULL) a unit is
 * HL_PEAK_ROWS rows of one image, with one image it is HL_PEAK_FLAT
 * consecutive int4 of its accumulator (a unit need not start a row: each
 * int4 finds its row).  A step of a unit is HL_PEAK_LOADS int4 per thread,
 * loaded at once (streaming loads) and compared with the threshold; an int4 holding
 * a bin above it -- rare -- is noted in shared memory, and a step that
 * noted any (one barrier tells) applies the peak rule to its notes.  The
 * loop keeps few registers, so HL_PEAK_CTAS_PER_SM CTAs fit an SM and many
 * loads are in flight. */
__global__ void __launch_bounds__(HL_PEAK_THREADS, HL_PEAK_CTAS_PER_SM) hl_peaks_kernel(hl_peak_args a)
{
    __shared__ unsigned s_note[HL_PEAK_LOADS * HL_PEAK_THREADS];   /* step offset << 4 | bins */
    __shared__ int s_nnote;
    const int q4 = a.Tp >> 2;
    const int tid = (int)threadIdx.x;
    if (tid == 0)
        s_nnote = 0;
    __syncthreads();
    hl_pdl_begin();
    if (a.cand.e) {
        const int nc = *a.cand.count;
        if (nc <= a.cand.cap) {
            for (int j = blockIdx.x * HL_PEAK_THREADS + tid; j < nc;
                 j += gridDim.x * HL_PEAK_THREADS) {
                const unsigned long long e = a.cand.e[j];
                const int img = (int)(e >> 32);
                const unsigned idx = (unsigned)e;
                const int row = (int)(idx / (unsigned)a.T), k = (int)(idx % (unsigned)a.T);
                const hl_peak_img &im = a.chunks ? a.imgs[img] : a.img0;
                if (row < im.R)
                    peak_bin(im.acc + (size_t)row * a.Tp + k, im.keys, im.ncand, im.R, im.cap,
                             a.T, a.Tp, row, k, a.status);
            }
            return;
        }
    }
    for (int c = blockIdx.x; c < a.nchunks; c += gridDim.x) {
        /* the unit: n int4 of image img from (row_lo, int4 column col_lo)
         * on; only what the loop needs stays in registers */
        int img = 0, row_lo, col_lo, n, thr;
        const int4 *src;
        if (a.chunks) {
            const int2 ch = a.chunks[c];
            const hl_peak_img &im = a.imgs[ch.x];
            img = ch.x;
            row_lo = ch.y;
            col_lo = 0;
            n = (min(ch.y + HL_PEAK_ROWS, im.R) - ch.y) * q4;
            thr = im.threshold;
            src = reinterpret_cast<const int4 *>(im.acc) + (size_t)row_lo * q4;
        } else {
            /* the host keeps R * Tp / 4 below 2^32 */
            const unsigned e_lo = (unsigned)c * HL_PEAK_FLAT;
            row_lo = (int)(e_lo / (unsigned)q4);
            col_lo = (int)(e_lo - (unsigned)row_lo * (unsigned)q4);
            n = (int)min((unsigned)HL_PEAK_FLAT, (unsigned)a.img0.R * (unsigned)q4 - e_lo);
            thr = a.img0.threshold;
            src = reinterpret_cast<const int4 *>(a.img0.acc) + e_lo;
        }
        for (int l0 = 0; l0 < n; l0 += HL_PEAK_LOADS * HL_PEAK_THREADS) {
            int4 v4[HL_PEAK_LOADS];
#pragma unroll
            for (int u = 0; u < HL_PEAK_LOADS; u++) {
                const int l = l0 + u * HL_PEAK_THREADS + tid;
                v4[u] = (l < n) ? __ldcs(src + l) : make_int4(0, 0, 0, 0);
            }
            bool noted = false;
#pragma unroll
            for (int u = 0; u < HL_PEAK_LOADS; u++) {
                const unsigned bits = (unsigned)(v4[u].x > thr) |
                                      ((unsigned)(v4[u].y > thr) << 1) |
                                      ((unsigned)(v4[u].z > thr) << 2) |
                                      ((unsigned)(v4[u].w > thr) << 3);
                if (bits) {
                    s_note[atomicAdd(&s_nnote, 1)] =
                        ((unsigned)(u * HL_PEAK_THREADS + tid) << 4) | bits;
                    noted = true;
                }
            }
            if (__syncthreads_or(noted)) {
                const int32_t *acc = a.chunks ? a.imgs[img].acc : a.img0.acc;
                unsigned long long *keys = a.chunks ? a.imgs[img].keys : a.img0.keys;
                int *ncand = a.chunks ? a.imgs[img].ncand : a.img0.ncand;
                const int R = a.chunks ? a.imgs[img].R : a.img0.R;
                const int cap = a.chunks ? a.imgs[img].cap : a.img0.cap;
                const int nn = s_nnote;
                /* a note per bin of the noted int4 */
                for (int j = tid; j < 4 * nn; j += HL_PEAK_THREADS) {
                    const unsigned e = s_note[j >> 2];
                    const int q = j & 3;
                    if (!((e >> q) & 1u))
                        continue;
                    const int t = col_lo + l0 + (int)(e >> 4);
                    const int dr = t / q4;
                    const int row = row_lo + dr, k = (t - dr * q4) * 4 + q;
                    if (k < a.T)
                        peak_bin(acc + (size_t)row * a.Tp + k, keys, ncand, R, cap, a.T, a.Tp,
                                 row, k, a.status);
                }
                __syncthreads();
                if (tid == 0)
                    s_nnote = 0;
                __syncthreads();
            }
        }
    }
}

cudaError_t hl_launch_peaks(const hl_peak_args *a, cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = std::max(1, std::min(a->nchunks, sms * HL_PEAK_CTAS_PER_SM));
    return hl_launch_pdl(hl_peaks_kernel, dim3(blocks), dim3(HL_PEAK_THREADS), 0, s, false, *a);
}

/* ------------------------------------------------------------------ */
/* finalize                                                             */

struct FinSmem {
    unsigned long long keys[FIN_CHUNK];
    unsigned long long sorted[FIN_CHUNK];
    float ang[FIN_CHUNK];
    int dist[FIN_CHUNK];
    int votes[FIN_CHUNK];
    /* earlier similar candidates; rows padded to 33 words so that threads
     * on consecutive candidates hit different banks */
    unsigned pred[FIN_CHUNK][FIN_CHUNK / 32 + 1];
    unsigned removed[FIN_CHUNK / 32];
    unsigned alive[FIN_CHUNK / 32];  /* kept candidates */
    int surv[FIN_CHUNK];
    float sang[FIN_SCACHE];
    int sdist[FIN_SCACHE];
    int hist[256];
    int misc[8];
};

/* The merge predicate, okano_3_0/HoughLine.cu:909-920, for an earlier line
 * (ai, di) and a later one (aj, dj): the angle test is in float, the
 * wrap-around angle M_PI - ai - aj in double, rounded to float.  The float
 * estimate (pi_f - ai) - aj is within 4e-7 of that value (pi_f is 8.7e-8 from
 * pi, two roundings of at most 1.2e-7 for operands below 2*pi, the final
 * rounding is below 4e-9 near the threshold), so the double form -- slow on
 * this GPU -- runs only when the estimate lies within 1e-6 of thresang. */
/* the exact wrap-around test (double), kept out of line so that it is only
 * ever executed, never evaluated speculatively */
static __device__ __noinline__ bool wrap_exact(float ai, float aj,
                                               float thresang)
{
    double t = __dsub_rn(__dsub_rn(3.14159265358979323846, (double)ai),
                         (double)aj);
    return __double2float_rn(fabs(t)) < thresang;
}

__device__ __forceinline__ bool similar(float ai, int di, float aj, int dj,
                                        int thresdis, float thresang)
{
    /* evaluated without short-circuit branches; only the rare ambiguous
     * wrap-around case branches */
    const bool same = (abs(di - dj) < thresdis) &
                      (fabsf(__fsub_rn(ai, aj)) < thresang);
    const bool near = abs(di + dj) < thresdis;
    const float est = fabsf(__fsub_rn(__fsub_rn(3.14159265f, ai), aj));
    const bool lo = est < thresang - 1e-6f, hi = est > thresang + 1e-6f;
    bool wrap = near & lo;
    if (near & !lo & !hi)
        wrap = wrap_exact(ai, aj, thresang);
    return same | wrap;
}

/* Reference decode, okano_3_0/HoughLine.cu:882-897. */
__device__ __forceinline__ void decode(unsigned long long key, int T,
                                       int rho_min, int off, float scale,
                                       double detheta, float *angle,
                                       int *distance, int *votes)
{
    const unsigned idx = ~(unsigned)(key & 0xffffffffu);
    const int row = (int)(idx / (unsigned)T), k = (int)(idx % (unsigned)T);
    const int rho = row + rho_min;
    const int ref_idx = (rho + off + 1) * (T + 2) + k + 1;
    const int rr = __float2int_rz(__fmul_rn(__int2float_rn(ref_idx), scale)) - 1;
    const int theta = ref_idx - (rr + 1) * (T + 2) - 1;
    *angle = __double2float_rn(__dmul_rn((double)theta, detheta));
    const int rel = rr - off;
    const float half = (rr >= 0) ? -0.5f : 0.5f;
    *distance = __float2int_rz(__fsub_rn(__int2float_rn(rel), half));
    *votes = (int)(key >> 32);
}

/* Predecessor bitmask of a sorted, decoded chunk of m candidates: bit j of
 * pred[i][j / 32] <=> j < i and similar(j, i).  Only the words holding some
 * j < i are built: entry (i, wd) for 32 wd < i, enumerated word by word.
 * Four adjacent threads share an entry (8 tests each, OR-ed by shuffles);
 * the threads of a warp mostly share wd and read the word's candidates with
 * broadcast loads.  Of nsub CTAs (a cluster) CTA sub takes every nsub-th
 * entry, so the CTAs share the work evenly; pred may be another CTA's
 * shared memory of the cluster. */
__device__ __forceinline__ void build_pred(const FinSmem &sm, int m, const hl_final_args &a,
                                           int sub, int nsub,
                                           unsigned (*pred)[FIN_CHUNK / 32 + 1])
{
    const int W = (m + 31) >> 5;
    int nent = 0;
    for (int wd = 0; wd < W; wd++)
        nent += max(0, m - 32 * wd - 1);
    const int q = threadIdx.x & 3;
    const int estep = (int)(blockDim.x >> 2) * nsub;
    /* a whole number of passes: every lane of a warp runs the same trips */
    const int span = (nent + estep - 1) / estep * estep;
    for (int en = (int)(threadIdx.x >> 2) * nsub + sub; en < span; en += estep) {
        unsigned bits = 0u;
        int i = 0, wd = 0, jn = 0;
        if (en < nent) {
            int rem = en;
            while (rem >= m - 32 * wd - 1) {
                rem -= m - 32 * wd - 1;
                wd++;
            }
            i = 32 * wd + 1 + rem;
            jn = min(32, i - (wd << 5));
        }
        {
            /* every lane runs the same 8 tests (invalid ones masked
             * afterwards), so the rare exact wrap-around test is a
             * warp-uniform branch */
            const int j0 = wd << 5;
            const float ai = sm.ang[i];
            const int di = sm.dist[i];
#pragma unroll
            for (int b = 8 * q; b < 8 * q + 8; b++) {
                const int j = min(j0 + b, m - 1);
                const float aj = sm.ang[j];
                const int dj = sm.dist[j];
                const bool same = (abs(dj - di) < a.thresdis) &
                                  (fabsf(__fsub_rn(aj, ai)) < a.thresang);
                const bool near = abs(dj + di) < a.thresdis;
                const float est = fabsf(__fsub_rn(__fsub_rn(3.14159265f, aj), ai));
                const bool lo = est < a.thresang - 1e-6f;
                const bool hi = est > a.thresang + 1e-6f;
                bool wrap = near & lo;
                const bool amb = near & !lo & !hi & (b < jn);
                if (__any_sync(FULL, amb)) {
                    if (amb)
                        wrap = wrap_exact(aj, ai, a.thresang);
                }
                bits |= (unsigned)((same | wrap) & (b < jn)) << b;
            }
        }
        bits |= __shfl_xor_sync(FULL, bits, 1);
        bits |= __shfl_xor_sync(FULL, bits, 2);
        if (en < nent && q == 0)
            pred[i][wd] = bits;
    }
}

/* Rank sort of keys[0, m) into sorted[] (descending): keys are unique (the
 * bin index is part of every key), so a key's rank is the number of larger
 * keys.  tpk consecutive threads (a power of two, as many as the threads
 * allow) rank one key, each against every tpk-th key, then sum by shuffles.
 * Keys [k_lo, k_hi) are ranked by threads [0, nthr); out[d] receives them
 * for d < ndst (several CTAs' arrays of a cluster). */
__device__ __forceinline__ void rank_keys(const unsigned long long *keys, int m, int k_lo,
                                          int k_hi, int nthr,
                                          unsigned long long *const *out, int ndst)
{
    const int tid = threadIdx.x;
    const int mk = k_hi - k_lo;
    if (mk <= 0)
        return;
    int tpk = 1;
    while (tpk < 32 && 2 * tpk * mk <= nthr)
        tpk <<= 1;
    const int per = nthr / tpk;
    const int part = tid & (tpk - 1);
    for (int i0 = 0; i0 < mk; i0 += per) {
        const int i = k_lo + i0 + tid / tpk;
        const bool have = i < k_hi;
        const unsigned long long ki = have ? keys[i] : 0ull;
        int rank = 0;
        if (have) {
            int j = part;
            for (; j + 3 * tpk < m; j += 4 * tpk)
                rank += (keys[j] > ki) + (keys[j + tpk] > ki) + (keys[j + 2 * tpk] > ki) +
                        (keys[j + 3 * tpk] > ki);
            for (; j < m; j += tpk)
                rank += keys[j] > ki;
        }
        for (int o = tpk >> 1; o > 0; o >>= 1)
            rank += __shfl_xor_sync(FULL, rank, o);
        if (have && part == 0)
            for (int d = 0; d < ndst; d++)
                out[d][rank] = ki;
    }
}

/* The greedy pass and the output of one sorted, decoded chunk whose
 * predecessor bitmask and `removed` words are built; S lines are already
 * written.  Returns the number of lines this chunk adds. */
__device__ int greedy_chunk(FinSmem &sm, const hl_final_img &im, int m, int K, int S)
{
    const int tid = threadIdx.x;
    const int W = (m + 31) >> 5;
    /* The greedy pass of okano_3_0/HoughLine.cu:900-927 keeps candidate i
     * iff it was not removed by an earlier chunk and no earlier kept
     * candidate is similar to it.  One warp resolves it a 32-candidate word
     * at a time, in order: lane j of word w (candidate i = 32 w + j) is
     * dropped by a kept candidate of an earlier word (its predecessor words
     * against the kept bits, all loads independent), then the word is
     * settled in rounds -- a candidate whose earlier in-word predecessors
     * are all decided is kept iff none of them is kept; each round settles
     * at least the lowest undecided lane, in practice one or two rounds
     * settle the word. */
    if (tid < 32) {
        const int lane = tid;
        if (lane >= W)
            sm.alive[lane] = 0u;   /* words past the chunk keep nobody */
        __syncwarp();
        for (int w = 0; w < W; w++) {
            const int i = 32 * w + lane;
            const bool valid = i < m;
            unsigned kill = valid ? (sm.removed[w] >> lane) & 1u : 1u;
            unsigned pin = 0u;
            if (valid) {
                for (int v = 0; v < w; v++)
                    kill |= sm.pred[i][v] & sm.alive[v];
                /* the in-word entry holds bits below the lane only (none
                 * was built for lane 0) */
                pin = lane ? sm.pred[i][w] & ((1u << lane) - 1u) : 0u;
            }
            unsigned und = __ballot_sync(FULL, kill == 0u);
            unsigned alive = 0u;
            while (und) {
                const bool in = (und >> lane) & 1u;
                const unsigned ready = __ballot_sync(FULL, in && !(pin & und));
                alive |= __ballot_sync(FULL, ((ready >> lane) & 1u) && !(pin & alive));
                und &= ~ready;
            }
            if (lane == 0)
                sm.alive[w] = alive;
            __syncwarp();
        }
    }
    __syncthreads();
    /* survivors in rank order, at most room of them */
    {
        const int room = K - S;
        for (int i = tid; i < m; i += blockDim.x) {
            const int iw = i >> 5;
            const unsigned al = sm.alive[iw];
            if ((al >> (i & 31)) & 1u) {
                int q = __popc(al & ((1u << (i & 31)) - 1u));
                for (int w = 0; w < iw; w++)
                    q += __popc(sm.alive[w]);
                if (q < room)
                    sm.surv[q] = i;
            }
        }
        if (tid < 32) {
            int c = __popc(sm.alive[tid]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                c += __shfl_xor_sync(FULL, c, o);
            if (tid == 0)
                sm.misc[3] = min(c, room);
        }
    }
    __syncthreads();
    const int ns = sm.misc[3];
    for (int q = tid; q < ns; q += blockDim.x) {
        const int i = sm.surv[q];
        const int o = S + q;
        hl_line L;
        L.angle = sm.ang[i];
        L.distance = sm.dist[i];
        L.votes = sm.votes[i];
        im.lines[o] = L;
        if (o < FIN_SCACHE) {
            sm.sang[o] = L.angle;
            sm.sdist[o] = L.distance;
        }
    }
    __syncthreads();
    return ns;
}

/* thread 0 after the last chunk: the line count, the candidate counter
 * cleared for the next call, overflow and status reporting */
__device__ void finalize_report(const hl_final_args &a, const hl_final_img &im, int S,
                                int ncand_raw)
{
    const int K = a.linesmax;
    const int cnt = (K > 0) ? S : K;
    if (im.count_out)
        *im.count_out = cnt;
    *im.ncand = 0;
    if (ncand_raw > im.cap)
        atomicOr(a.status, HL_ST_CAND_OVERFLOW);
    if (a.hdr) {   /* one image: report and clear the status word */
        int st = *a.status;
        if (ncand_raw > im.cap)
            st |= HL_ST_CAND_OVERFLOW;
        a.hdr->count = cnt;
        a.hdr->status = st;
        a.hdr->ncand = ncand_raw;
        *a.status = 0;
    }
}

/* One CTA, one image: the whole tail (okano_3_0/HoughLine.cu:837-948) in
 * chunks of FIN_CHUNK keys. */
__device__ void finalize_cta(const hl_final_args &a, const hl_final_img &im, float scale,
                             FinSmem &sm)
{
    const int tid = threadIdx.x;
    const int ncand_raw = *im.ncand;
    const int n = min(ncand_raw, im.cap);
    const int K = a.linesmax;
    const int off = (im.ref_numrho - 1) / 2;
    int S = 0;          /* survivors written so far */
    int taken = 0;
    unsigned long long upper = ~0ull;

    while (taken < n && S < K) {
        const int m = min(FIN_CHUNK, n - taken);
        if (n <= FIN_CHUNK) {
            for (int i = tid; i < m; i += blockDim.x)
                sm.keys[i] = im.keys[i];
        } else {
            /* MSD radix select of the m-th largest key below `upper` */
            unsigned long long prefix = 0, pmask = 0;
            int need = m;
            for (int d = 7; d >= 0; d--) {
                for (int i = tid; i < 256; i += blockDim.x)
                    sm.hist[i] = 0;
                __syncthreads();
                for (int i = tid; i < n; i += blockDim.x) {
                    unsigned long long kk = im.keys[i];
                    if (kk < upper && (kk & pmask) == prefix)
                        atomicAdd(&sm.hist[(kk >> (8 * d)) & 255], 1);
                }
                __syncthreads();
                if (tid == 0) {
                    int c = 0, bsel = 0;
                    for (int bb = 255; bb >= 0; bb--) {
                        if (c + sm.hist[bb] >= need) {
                            bsel = bb;
                            break;
                        }
                        c += sm.hist[bb];
                    }
                    sm.misc[0] = bsel;
                    sm.misc[1] = need - c;
                }
                __syncthreads();
                prefix |= (unsigned long long)sm.misc[0] << (8 * d);
                pmask |= 255ull << (8 * d);
                need = sm.misc[1];
                __syncthreads();
            }
            if (tid == 0)
                sm.misc[2] = 0;
            __syncthreads();
            for (int i = tid; i < n; i += blockDim.x) {
                unsigned long long kk = im.keys[i];
                if (kk < upper && kk >= prefix) {
                    int pos = atomicAdd(&sm.misc[2], 1);
                    if (pos < FIN_CHUNK)
                        sm.keys[pos] = kk;
                }
            }
            __syncthreads();
        }
        __syncthreads();
        {
            unsigned long long *dst = sm.sorted;
            rank_keys(sm.keys, m, 0, m, blockDim.x, &dst, 1);
        }
        __syncthreads();
        taken += m;
        upper = sm.sorted[m - 1];

        /* decode; drop candidates similar to a survivor of an earlier chunk */
        for (int i = tid; i < 32; i += blockDim.x)
            sm.removed[i] = 0u;
        __syncthreads();
        for (int i = tid; i < m; i += blockDim.x) {
            float ang;
            int dist, vts;
            decode(sm.sorted[i], a.T, im.rho_min, off, scale, a.detheta, &ang,
                   &dist, &vts);
            sm.ang[i] = ang;
            sm.dist[i] = dist;
            sm.votes[i] = vts;
            bool dead = false;
            for (int q = 0; q < S && !dead; q++) {
                float qa;
                int qd;
                if (q < FIN_SCACHE) {
                    qa = sm.sang[q];
                    qd = sm.sdist[q];
                } else {
                    qa = im.lines[q].angle;
                    qd = im.lines[q].distance;
                }
                dead = similar(qa, qd, ang, dist, a.thresdis, a.thresang);
            }
            if (dead)
                atomicOr(&sm.removed[i >> 5], 1u << (i & 31));
        }
        __syncthreads();
        build_pred(sm, m, a, 0, 1, sm.pred);
        __syncthreads();
        S += greedy_chunk(sm, im, m, K, S);
    }
    if (tid == 0)
        finalize_report(a, im, S, ncand_raw);
}

__global__ void __launch_bounds__(FIN_THREADS)
hl_finalize_kernel(hl_final_args a, float scale)
{
    extern __shared__ __align__(16) unsigned char fin_raw[];
    FinSmem &sm = *reinterpret_cast<FinSmem *>(fin_raw);
    hl_pdl_begin();
    const hl_final_img im = a.imgs ? a.imgs[blockIdx.x] : a.img0;  /* CTA = image */
    finalize_cta(a, im, scale, sm);
}

#define FIN_CLUSTER 8

/* One image on a cluster of FIN_CLUSTER CTAs (one per SM) when its peaks
 * fit one chunk: every CTA loads the keys, ranks an eighth of them into
 * every CTA's sorted[] (distributed shared memory), decodes all of them and
 * builds an eighth of the predecessor words into CTA 0's bitmask; after the
 * cluster barrier CTA 0 alone runs the greedy pass.  With more peaks than a
 * chunk CTA 0 runs finalize_cta and the others leave at once (no shared
 * memory of another CTA is touched in that case). */
__global__ void __cluster_dims__(FIN_CLUSTER, 1, 1) __launch_bounds__(FIN_THREADS)
hl_finalize_cluster_kernel(hl_final_args a, float scale)
{
    extern __shared__ __align__(16) unsigned char fin_raw[];
    FinSmem &sm = *reinterpret_cast<FinSmem *>(fin_raw);
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int tid = threadIdx.x;
    hl_pdl_begin();
    const hl_final_img im = a.img0;
    const int ncand_raw = *im.ncand;
    const int n = min(ncand_raw, im.cap);
    const int K = a.linesmax;
    if (n > FIN_CHUNK || n == 0 || K <= 0) {
        if (rank == 0)
            finalize_cta(a, im, scale, sm);
        return;
    }
    const int m = n;
    for (int i = tid; i < m; i += blockDim.x)
        sm.keys[i] = im.keys[i];
    __syncthreads();
    {
        unsigned long long *dst[FIN_CLUSTER];
#pragma unroll
        for (int d = 0; d < FIN_CLUSTER; d++)
            dst[d] = cl.map_shared_rank(sm.sorted, d);
        rank_keys(sm.keys, m, m * rank / FIN_CLUSTER, m * (rank + 1) / FIN_CLUSTER,
                  blockDim.x, dst, FIN_CLUSTER);
    }
    cl.sync();
    const int off = (im.ref_numrho - 1) / 2;
    for (int i = tid; i < m; i += blockDim.x) {
        float ang;
        int dist, vts;
        decode(sm.sorted[i], a.T, im.rho_min, off, scale, a.detheta, &ang, &dist, &vts);
        sm.ang[i] = ang;
        sm.dist[i] = dist;
        sm.votes[i] = vts;
    }
    if (rank == 0)
        for (int i = tid; i < 32; i += blockDim.x)
            sm.removed[i] = 0u;
    __syncthreads();
    build_pred(sm, m, a, rank, FIN_CLUSTER,
               reinterpret_cast<unsigned (*)[FIN_CHUNK / 32 + 1]>(
                   cl.map_shared_rank(&sm.pred[0][0], 0)));
    cl.sync();
    if (rank != 0)
        return;
    const int S = greedy_chunk(sm, im, m, K, 0);
    if (tid == 0)
        finalize_report(a, im, S, ncand_raw);
}

cudaError_t hl_launch_finalize(const hl_final_args *a, int nimg, cudaStream_t s)
{
    const size_t smem = sizeof(FinSmem);
    const float scale = (float)(1.0 / (a->T + 2));   /* :882-883 */
    cudaError_t e;
    if (nimg == 1 && !a->imgs) {
        /* one image: a cluster spreads the sort and the bitmask */
        e = cudaFuncSetAttribute(hl_finalize_cluster_kernel,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
        return hl_launch_pdl(hl_finalize_cluster_kernel, dim3(FIN_CLUSTER), dim3(FIN_THREADS),
                             smem, s, false, *a, scale);
    }
    e = cudaFuncSetAttribute(hl_finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess)
        return e;
    return hl_launch_pdl(hl_finalize_kernel, dim3(nimg), dim3(FIN_THREADS), smem, s, false, *a,
                         scale);
}

/* ---- one small image in one launch ----------------------------------------
 * A cluster of Tp / 32 CTAs (1024 threads each), CTA c owning theta slice c
 * and the whole rho range of it in shared memory (R rows x 32 columns plus a
 * dump row), so no accumulator goes to HBM:
 *   1. CTA c compacts the ROI rows [c h / C, (c + 1) h / C) into its part of
 *      one global point list (ROI-local float (x, y); a count pass, the
 *      counts exchanged through distributed shared memory after a cluster
 *      barrier, then a write pass at the CTA's offset from the first pass's
 *      edge masks, kept in registers when a thread has one batch of chunks;
 *      the order inside the list is free, the counts do not depend on it);
 *   2. after a second cluster barrier every CTA votes every point of the list
 *      into its slice with the vote kernel's diagonal schedule (the vote rule
 *      of okano_3_0/HoughLine.cu:86-130, exact float -> integer conversion);
 *   3. after a third barrier the peak rule (:168-213, bounds-checked, zero
 *      outside the accumulator) runs on the slice in shared memory, the
 *      neighbours across a slice edge read from the next CTA's shared memory
 *      (distributed shared memory loads), peaks appended as keys;
 *   4. after a fourth barrier (no CTA reads another's slice any more) CTA 0
 *      reuses its shared memory for the tail (rank, decode, merge, truncate:
 *      finalize_cta) and writes the result.
 * The four cluster barriers are the only waits. */
#define SMALL_THREADS 1024

/* 4-bit mask of the bytes of w equal to 0xFF (bit b = byte b) */
__device__ __forceinline__ uint32_t eq255_mask4(uint32_t w)
{
    const uint32_t m = __vcmpeq4(w, 0xffffffffu) & 0x80808080u;
    return ((m >> 7) | (m >> 14) | (m >> 21) | (m >> 28)) & 15u;
}

static inline size_t small_smem(int R)
{
    const size_t acc = (size_t)(R + 1) * HL_SLICE * sizeof(int);
    return acc > sizeof(FinSmem) ? acc : sizeof(FinSmem);
}

int hl_small_fits(int T, int Tp, int R)
{
    const int C = Tp / HL_SLICE;
    return T > 0 && C >= 1 && C <= HL_SMALL_MAX_CTAS && R > 0 &&
           small_smem(R) <= 227u * 1024u;
}

/* Edge masks of this thread's four 16-pixel chunks c, c + SMALL_THREADS, ...
 * of the rows [y0, ...) (bit b = pixel x + b is 255; 0 past nch) */
__device__ __forceinline__ void small_chunk_masks(const hl_roi &roi, int y0, int cw, int nch,
                                                  int w, int c, uint32_t mm[4])
{
    uint4 v[4];
    bool vec[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int cc = c + u * SMALL_THREADS;
        const int y = y0 + cc / cw, x = (cc % cw) * 16;
        const uint8_t *pp = roi.base + (size_t)y * roi.pitch + x;
        vec[u] = cc < nch && x + 16 <= w && (((uintptr_t)pp) & 15u) == 0;
        v[u] = vec[u] ? __ldcs(reinterpret_cast<const uint4 *>(pp)) : make_uint4(0, 0, 0, 0);
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int cc = c + u * SMALL_THREADS;
        uint32_t m = 0;
        if (vec[u]) {
            m = eq255_mask4(v[u].x) | (eq255_mask4(v[u].y) << 4) |
                (eq255_mask4(v[u].z) << 8) | (eq255_mask4(v[u].w) << 12);
        } else if (cc < nch) {
            const int y = y0 + cc / cw, x = (cc % cw) * 16;
            const uint8_t *pp = roi.base + (size_t)y * roi.pitch + x;
            const int lim = min(16, w - x);
            for (int b = 0; b < lim; b++)
                m |= (uint32_t)(pp[b] == 255) << b;
        }
        mm[u] = m;
    }
}

template <bool UNIT>
__global__ void __launch_bounds__(SMALL_THREADS, 1)
hl_small_kernel(hl_small_args a)
{
    extern __shared__ __align__(16) unsigned char small_raw[];
    int *acc = reinterpret_cast<int *>(small_raw);
    __shared__ int s_cnt, s_wr;
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks(), rank = (int)cl.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = SMALL_THREADS / 32;
    const int w = a.roi.w, h = a.roi.h;

    /* 1. compaction of this CTA's rows in two passes over 16-pixel chunks
     * (four 16-byte loads in flight per thread; byte loads where a chunk is
     * unaligned or runs past the ROI's right edge): count, exchange the
     * counts across the cluster, then write the points at this CTA's offset
     * of one contiguous list (the second pass reads the rows from L2).  The
     * slice is cleared meanwhile. */
    for (int i = tid; i < (a.R + 1) * HL_SLICE; i += SMALL_THREADS)
        acc[i] = 0;
    if (tid == 0) {
        s_cnt = 0;
        s_wr = 0;
    }
    __syncthreads();
    const int y0 = (int)((long long)h * rank / C), y1 = (int)((long long)h * (rank + 1) / C);
    const int cw = (w + 15) >> 4;
    const int nch = (y1 - y0) * cw;
    int mycnt = 0;
    const bool one_batch = nch <= 4 * SMALL_THREADS;   /* masks kept in registers */
    uint32_t kept[4] = {0u, 0u, 0u, 0u};
    for (int c0 = 0; c0 < nch; c0 += 4 * SMALL_THREADS) {
        uint32_t mm[4];
        small_chunk_masks(a.roi, y0, cw, nch, w, c0 + tid, mm);
        mycnt += __popc(mm[0]) + __popc(mm[1]) + __popc(mm[2]) + __popc(mm[3]);
        if (one_batch) {
#pragma unroll
            for (int u = 0; u < 4; u++)
                kept[u] = mm[u];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        mycnt += __shfl_xor_sync(FULL, mycnt, o);
    if (lane == 0 && mycnt)
        atomicAdd(&s_cnt, mycnt);
    cl.sync();
    int start = 0, ntot = 0;
    for (int r = 0; r < C; r++) {
        const int n = *cl.map_shared_rank(&s_cnt, r);
        start += r < rank ? n : 0;
        ntot += n;
    }
    for (int c0 = 0; c0 < nch; c0 += 4 * SMALL_THREADS) {
        uint32_t mm[4];
        if (one_batch) {
#pragma unroll
            for (int u = 0; u < 4; u++)
                mm[u] = kept[u];
        } else {
            small_chunk_masks(a.roi, y0, cw, nch, w, c0 + tid, mm);
        }
        const int cnt = __popc(mm[0]) + __popc(mm[1]) + __popc(mm[2]) + __popc(mm[3]);
        int pos = cnt ? start + atomicAdd(&s_wr, cnt) : 0;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int c = c0 + tid + u * SMALL_THREADS;
            const float y = (float)(y0 + c / cw);
            const int x = (c % cw) * 16;
            for (uint32_t m = mm[u]; m; m &= m - 1)
                a.pts[pos++] = make_float2((float)(x + __ffs(m) - 1), y);
        }
    }
    __threadfence();
    cl.sync();

    /* 2. every point voted into this slice, rounds of 8 points, four
     * rounds' loads in flight per warp (the points come from L2) */
    const int k0 = rank * HL_SLICE;
    DiagTab tab;
    diag_table(tab, a.cosv + k0, a.sinv + k0, (unsigned)__cvta_generic_to_shared(acc), lane);
    const f2x ir = f2_pack(a.irho, a.irho);
    const int p = lane & 7;
    for (int g0 = warp * 8; g0 < ntot; g0 += 4 * nwarps * 8) {
        float2 q[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int gi = g0 + u * nwarps * 8 + p;
            q[u] = gi < ntot ? a.pts[gi] : make_float2(1e30f, 0.0f);
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (g0 + u * nwarps * 8 < ntot)
                diag_point<UNIT, CV_SIGN>(q[u].x, q[u].y, tab, ir, RHO_MAGIC_BITS + a.rho_min,
                                          (unsigned)a.R);
    }
    cl.sync();

    /* 3. peaks of the slice: v > thr, v > W, v >= E, v > N, v >= S */
    const int *accL = rank > 0 ? cl.map_shared_rank(acc, rank - 1) : nullptr;
    const int *accR = rank + 1 < C ? cl.map_shared_rank(acc, rank + 1) : nullptr;
    const hl_final_img &im = a.fin.img0;
    const int4 *acc4 = reinterpret_cast<const int4 *>(acc);
    const int n4 = a.R * (HL_SLICE / 4);
    /* a uniform trip count for every warp (the warp collectives below) */
    for (int b4 = 0; b4 < n4; b4 += SMALL_THREADS) {
        const int i4 = b4 + tid;
        const int4 q4 = i4 < n4 ? acc4[i4] : make_int4(0, 0, 0, 0);
        const int mx = max(max(q4.x, q4.y), max(q4.z, q4.w));
        unsigned found = 0;   /* bit e: bin 4 i4 + e is a peak */
        if (i4 < n4 && mx > a.threshold) {
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int i = 4 * i4 + e;
                const int row = i >> 5, j = i & 31, k = k0 + j;
                const int v = e == 0 ? q4.x : e == 1 ? q4.y : e == 2 ? q4.z : q4.w;
                if (k < a.T && v > a.threshold) {
                    const int W = j > 0 ? acc[i - 1] : (accL ? accL[row * HL_SLICE + 31] : 0);
                    const int E = k + 1 >= a.T ? 0
                                  : (j < 31 ? acc[i + 1] : accR[row * HL_SLICE]);
                    const int N = row > 0 ? acc[i - HL_SLICE] : 0;
                    const int S = row + 1 < a.R ? acc[i + HL_SLICE] : 0;
                    if (v > W && v >= E && v > N && v >= S)
                        found |= 1u << e;
                }
            }
        }
        const int cnt = __popc(found);
        const unsigned any = __ballot_sync(FULL, cnt > 0);
        if (!any)
            continue;
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o)
                incl += t;
        }
        int base = 0;
        if (lane == 31)
            base = atomicAdd(im.ncand, incl);
        base = __shfl_sync(FULL, base, 31);
        int pos = base + incl - cnt;
        for (unsigned f = found; f; f &= f - 1) {
            const int e = __ffs(f) - 1;
            const int i = 4 * i4 + e;
            const int row = i >> 5, k = k0 + (i & 31);
            const int v = e == 0 ? q4.x : e == 1 ? q4.y : e == 2 ? q4.z : q4.w;
            if (pos < im.cap) {
                const unsigned idx = (unsigned)row * (unsigned)a.T + (unsigned)k;
                const_cast<unsigned long long *>(im.keys)[pos] =
                    ((unsigned long long)(unsigned)v << 32) | (unsigned)(~idx);
            }
            pos++;
        }
    }
    __threadfence();
    cl.sync();

    /* 4. the tail on CTA 0, in the shared memory the slice used */
    if (rank != 0)
        return;
    FinSmem &sm = *reinterpret_cast<FinSmem *>(small_raw);
    finalize_cta(a.fin, im, a.scale, sm);
}

cudaError_t hl_launch_small(const hl_small_args *a, cudaStream_t s)
{
    const int C = a->Tp / HL_SLICE;
    const size_t smem = small_smem(a->R);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C);
    cfg.blockDim = dim3(SMALL_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e;
    if (a->irho == 1.0f) {
        e = cudaFuncSetAttribute(hl_small_kernel<true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
        return cudaLaunchKernelEx(&cfg, hl_small_kernel<true>, *a);
    }
    e = cudaFuncSetAttribute(hl_small_kernel<false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    return cudaLaunchKernelEx(&cfg, hl_small_kernel<false>, *a);
}

/* acc[R][Tp] -> acc[R][T] */
__global__ void hl_to_tight_kernel(const int32_t *acc, int R, int T, int Tp,
                                   int32_t *out)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t total = (size_t)R * T;
    if (i >= total)
        return;
    size_t row = i / T, k = i % T;
    out[i] = acc[row * Tp + k];
}

cudaError_t hl_launch_to_tight(const int32_t *acc, int R, int T, int Tp,
                               int32_t *out, cudaStream_t s)
{
    size_t total = (size_t)R * T;
    hl_to_tight_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(acc, R, T,
                                                                     Tp, out);
    return cudaGetLastError();
}

/* acc[R][Tp] -> reference layout (T+2) x (ref_numrho+2) with zero border,
 * okano_3_0/HoughLine.cu:122-124. */
__global__ void hl_to_ref_kernel(const int32_t *acc, int R, int T, int Tp,
                                 int rho_min, int ref_numrho, int32_t *ref)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t total = (size_t)(T + 2) * (size_t)(ref_numrho + 2);
    if (i >= total)
        return;
    int prow = (int)(i / (T + 2)), pcol = (int)(i % (T + 2));
    int v = 0;
    int k = pcol - 1, row_ref = prow - 1;
    if (k >= 0 && k < T && row_ref >= 0 && row_ref < ref_numrho) {
        int rho = row_ref - (ref_numrho - 1) / 2;
        int row = rho - rho_min;
        if (row >= 0 && row < R)
            v = acc[(size_t)row * Tp + k];
    }
    ref[i] = v;
}

cudaError_t hl_launch_to_ref(const int32_t *acc, int R, int T, int Tp,
                             int rho_min, int ref_numrho, int32_t *ref,
                             cudaStream_t s)
{
    size_t total = (size_t)(T + 2) * (size_t)(ref_numrho + 2);
    hl_to_ref_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
        acc, R, T, Tp, rho_min, ref_numrho, ref);
    return cudaGetLastError();
}

/* acc[R][T] -> acc[R][Tp] (zero padding columns) */
__global__ void hl_from_tight_kernel(const int32_t *acc, int R, int T, int Tp,
                                     int32_t *out)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t total = (size_t)R * Tp;
    if (i >= total)
        return;
    size_t row = i / Tp, k = i % Tp;
    out[i] = (k < (size_t)T) ? acc[row * T + k] : 0;
}

cudaError_t hl_launch_from_tight(const int32_t *acc, int R, int T, int Tp,
                                 int32_t *out, cudaStream_t s)
{
    size_t total = (size_t)R * Tp;
    hl_from_tight_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
        acc, R, T, Tp, out);
    return cudaGetLastError();
}
