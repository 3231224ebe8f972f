/*
 * hl_window.cu -- the exact vote of the proposal-guided path.
 *
 * hl_select_kernel: one CTA per image reads the network's 90 x 128 logits,
 * keeps the candidates (local maxima, or every cell) above the cutoff and
 * the image's best top_m, falls back to the full method when the network
 * sees more likely lines than that (count and confidence tests), grows the
 * kept cells by the dilation and appends one window per cell.
 *
 * hl_window_vote_kernel: one CTA per window, a run of up to HL_WIN_RUN
 * marked coarse cells (t, r .. r1) at one theta cell.  A coarse cell (t, r)
 * owns the fine thetas k with floor(90 k / T) = t and the rho rows j with
 * floor(128 j / R) = r; the CTA votes the run's bins plus a one-bin halo with
 * the plain method's rule (okano_3_0/HoughLine.cu:86-130) from every point of
 * the tiles that can reach them, then applies the peak rule (:168-213) to the
 * owned bins with the halo as their neighbours (bins outside the accumulator
 * count 0).  Counts and neighbours are exact, so a reported peak is a peak of
 * the full accumulator with its exact vote count; windows own disjoint bins,
 * so no peak is reported twice.  Peaks go to the image's key list in the
 * plain path's format and the batched finalize ranks and merges them.
 */
#include "hl_device.cuh"
#include "hl_internal.h"
#include "hl_window.h"

#include <algorithm>

#define FULL 0xffffffffu

#define NCELL (HL_COARSE_T * HL_COARSE_R)

/* Is coarse cell i a local maximum of the logits (3 x 3 neighbourhood, ties
 * to the earlier cell in raster order)? */
__device__ __forceinline__ bool local_max(const float *z, int i)
{
    const int t = i / HL_COARSE_R, r = i % HL_COARSE_R;
    const float v = z[i];
    for (int dt = -1; dt <= 1; dt++) {
        const int tt = t + dt;
        if (tt < 0 || tt >= HL_COARSE_T)
            continue;
        for (int dr = -1; dr <= 1; dr++) {
            const int rr = r + dr;
            if ((dt == 0 && dr == 0) || rr < 0 || rr >= HL_COARSE_R)
                continue;
            const int j = tt * HL_COARSE_R + rr;
            const float u = z[j];
            if (u > v || (u == v && j < i))
                return false;
        }
    }
    return true;
}

/* Value level with at least `target` of the n candidate values cv above it
 * (bisection on the value; the block's threads count in parallel).  Returns
 * -inf when there are at most `target` candidates. */
__device__ float level_for(const float *cv, int n, int target, float *red, int *s_cnt)
{
    if (n <= target)
        return -3.0e38f;
    float mn = 3.0e38f, mx = -3.0e38f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        mn = fminf(mn, cv[i]);
        mx = fmaxf(mx, cv[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(FULL, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = mn;
        red[16 + (threadIdx.x >> 5)] = mx;
    }
    __syncthreads();
    float lo = red[0], hi = red[16];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
        lo = fminf(lo, red[w]);
        hi = fmaxf(hi, red[16 + w]);
    }
    lo -= 1.0f;   /* count(cv > lo) = n >= target */
    for (int it = 0; it < 24; it++) {
        const float mid = 0.5f * (lo + hi);
        __syncthreads();
        if (threadIdx.x == 0)
            *s_cnt = 0;
        __syncthreads();
        int c = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            c += cv[i] > mid;
        atomicAdd(s_cnt, c);
        __syncthreads();
        if (*s_cnt >= target)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

/* One CTA per image.  Candidates are the coarse cells (with nms: the local
 * maxima of the logits); selected are the candidates above the cutoff and
 * the image's top_m candidates, each grown by the dilation into windows.
 * The image falls back to the plain method when more than max_props
 * candidates clear the cutoff (a cluttered scene), or -- the confidence
 * test -- when the best candidate left out of the top_m is itself above
 * zconf: the network sees more likely lines than the budget covers. */
__global__ void __launch_bounds__(512)
hl_select_kernel(hl_select_args a)
{
    extern __shared__ float zs[];          /* [NCELL] logits, [NCELL] candidate values */
    float *cv = zs + NCELL;
    __shared__ unsigned mark[NCELL / 32];
    __shared__ int cnt, ncand, s_cnt;
    __shared__ float red[32];
    const int b = blockIdx.x;
    const float *z = a.logits + (size_t)b * NCELL;
    for (int i = threadIdx.x; i < NCELL; i += blockDim.x)
        zs[i] = z[i];
    for (int i = threadIdx.x; i < NCELL / 32; i += blockDim.x)
        mark[i] = 0u;
    if (threadIdx.x == 0) {
        cnt = 0;
        ncand = 0;
    }
    __syncthreads();
    int mine = 0;
    for (int i = threadIdx.x; i < NCELL; i += blockDim.x) {
        if (a.nms && !local_max(zs, i))
            continue;
        cv[atomicAdd(&ncand, 1)] = zs[i];
        mine += zs[i] > a.zcut;
    }
    atomicAdd(&cnt, mine);
    __syncthreads();
    const int nc = ncand;
    int fb = (cnt > a.max_props || a.force_fallback) ? 1 : 0;
    float level = a.zcut;
    if (!fb && a.top_m > 0) {
        level = fminf(level, level_for(cv, nc, a.top_m, red, &s_cnt));
        if (a.use_conf && nc > a.top_m) {
            /* the (top_m + 1)-th candidate lies above this level */
            const float next = level_for(cv, nc, a.top_m + 1, red, &s_cnt);
            if (next >= a.zconf)
                fb = 2;
        }
    }
    if (threadIdx.x == 0)
        a.fallback[b] = fb;
    if (fb)
        return;
    for (int i = threadIdx.x; i < NCELL; i += blockDim.x) {
        if (!(zs[i] > level) || (a.nms && !local_max(zs, i)))
            continue;
        const int t = i / HL_COARSE_R, r = i % HL_COARSE_R;
        for (int dt = -a.dil_t; dt <= a.dil_t; dt++) {
            const int tt = t + dt;
            if (tt < 0 || tt >= HL_COARSE_T)
                continue;
            for (int dr = -a.dil_r; dr <= a.dil_r; dr++) {
                const int rr = r + dr;
                if (rr < 0 || rr >= HL_COARSE_R)
                    continue;
                const int c = tt * HL_COARSE_R + rr;
                atomicOr(&mark[c >> 5], 1u << (c & 31));
            }
        }
    }
    __syncthreads();
    /* one window per run of marked cells along rho at one theta (a mask
     * word holds 32 consecutive rho cells of one theta cell), at most
     * HL_WIN_RUN cells: the run's points are read once for all its cells */
    for (int wd = threadIdx.x; wd < NCELL / 32; wd += blockDim.x) {
        unsigned m = mark[wd];
        if (m)
            atomicAdd(a.ncells, __popc(m));
        while (m) {
            const int bit = __ffs(m) - 1;
            const unsigned ones = ~(m >> bit);            /* the run ends at its first 0 */
            const int len = min(ones ? __ffs(ones) - 1 : 32 - bit, HL_WIN_RUN);
            m &= ~(((len == 32 ? 0u : (1u << len)) - 1u) << bit);
            const int c = wd * 32 + bit;
            const int q = atomicAdd(a.nwin, 1);
            if (q < a.cap)
                a.win[q] = make_int4(b, c / HL_COARSE_R, c % HL_COARSE_R,
                                     c % HL_COARSE_R + len - 1);
            else
                atomicOr(a.status, HL_ST_CAND_OVERFLOW);
        }
    }
}

cudaError_t hl_launch_select(const hl_select_args *a, int nimg, cudaStream_t s)
{
    const int smem = (int)(2 * NCELL * sizeof(float));
    cudaError_t e = cudaFuncSetAttribute(hl_select_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess)
        return e;
    hl_select_kernel<<<nimg, 512, smem, s>>>(*a);
    return cudaGetLastError();
}

/* fine range [lo, hi) of coarse index c of n coarse cells over m fine bins:
 * the bins j with floor(n j / m) = c */
__device__ __forceinline__ void fine_range(int c, int n, int m, int *lo, int *hi)
{
    *lo = (int)(((long long)c * m + n - 1) / n);
    *hi = (int)(((long long)(c + 1) * m + n - 1) / n);
}

/* The votes of one point into a window's haloed bins (nk thetas of
 * cos/sin s_c/s_s, nj rows from the row whose rho bits are `base`): the
 * plain method's rule (okano_3_0/HoughLine.cu:115-121) with the float ->
 * integer step by the window's conversion (CV_FLOOR / CV_CEIL: the magic
 * constant, see RHO_MAGIC; CV_EXACT: the conversion instruction).  The lane
 * starts at theta kk0 and walks the thetas round, so at a time the warp's
 * lanes vote about 32 / nk lanes per theta: points of one line (which
 * share a bin at its theta) collide in groups of that size, not 32. */
template <bool UNIT, int CV>
__device__ __forceinline__ void window_point(float x, float y, const float *s_c,
                                             const float *s_s, int nk, int kk0, int base,
                                             int nj, unsigned acc_base, float irho)
{
    int kk = kk0;
    for (int st = 0; st < nk; st++) {
        const float v = rho_f<UNIT>(x, y, s_c[kk], s_s[kk], irho);
        int j;
        if (CV == CV_FLOOR)
            j = __float_as_int(__fadd_rz(v, RHO_MAGIC)) - base;
        else if (CV == CV_CEIL)
            j = __float_as_int(__fadd_ru(v, RHO_MAGIC)) - base;
        else
            j = __float2int_rz(v) - base;
        if ((unsigned)j < (unsigned)nj)
            red_smem(acc_base + (unsigned)(kk * (nj + 1) + j) * 4u);
        if (++kk == nk)
            kk = 0;
    }
}

/* The points of the window's hit tiles: with the hit tiles listed (nhit of
 * them, at most HL_WIN_HITS), warp w takes hits w, w + 8, ... -- the hits of
 * a strip bunch in a few mask words, so taking whole mask words left most
 * warps idle -- else warp w takes mask words w, w + 8, ... */
template <bool UNIT, int CV>
__device__ __forceinline__ void window_tiles(const hl_vote_img &im, const unsigned *tmask,
                                             int ntl, const unsigned short *hits, int nhit,
                                             const float *s_c, const float *s_s, int nk,
                                             int base, int nj, unsigned acc_base, float irho)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    const int kk0 = lane % nk;
    if (nhit <= HL_WIN_HITS) {
        for (int h = warp; h < nhit; h += nw) {
            const int tl = hits[h];
            const int p0 = im.tile_off[tl], p1 = im.tile_off[tl + 1];
            for (int p = p0 + lane; p < p1; p += 32) {
                const float2 xy = im.pts[p];
                window_point<UNIT, CV>(xy.x, xy.y, s_c, s_s, nk, kk0, base, nj, acc_base,
                                       irho);
            }
        }
        return;
    }
    for (int wd = warp; wd < (ntl + 31) / 32; wd += nw) {
        unsigned m = tmask[wd];
        while (m) {
            const int tl = wd * 32 + __ffs(m) - 1;
            m &= m - 1;
            const int p0 = im.tile_off[tl], p1 = im.tile_off[tl + 1];
            for (int p = p0 + lane; p < p1; p += 32) {
                const float2 xy = im.pts[p];
                window_point<UNIT, CV>(xy.x, xy.y, s_c, s_s, nk, kk0, base, nj, acc_base,
                                       irho);
            }
        }
    }
}

/* float -> integer of the window's conversion (RHO_MAGIC), as bits */
template <int CV>
__device__ __forceinline__ int conv_bits(float v)
{
    if (CV == CV_FLOOR)
        return __float_as_int(__fadd_rz(v, RHO_MAGIC));
    if (CV == CV_CEIL)
        return __float_as_int(__fadd_ru(v, RHO_MAGIC));
    return __float2int_rz(v);
}

/* The common case, at most NK thetas (NK a compile-time bound): the
 * thetas' cos / sin and column addresses in registers, every lane votes its
 * point for theta 0, 1, ... with no branch -- a row outside the window
 * goes to the column's dump row nj (rows are nj + 1 apart), a theta past
 * the window's nk to a column of its own that nothing reads (cos = sin =
 * 0).  Warp w takes the listed hit tiles w, w + 8, ... */
template <bool UNIT, int CV, int NK>
__device__ __forceinline__ void window_tiles_nk(const hl_vote_img &im, const unsigned short *hits,
                                                int nhit, const float *s_c, const float *s_s,
                                                int base, int nj, unsigned acc_base, float irho)
{
    float c[NK], sn[NK];
    unsigned kb[NK];
#pragma unroll
    for (int k = 0; k < NK; k++) {
        c[k] = s_c[k];
        sn[k] = s_s[k];
        kb[k] = acc_base + (unsigned)(k * (nj + 1)) * 4u;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    for (int h = warp; h < nhit; h += nw) {
        const int tl = hits[h];
        const int p0 = im.tile_off[tl], p1 = im.tile_off[tl + 1];
        /* the next point's load issued before this one's votes */
        float2 nxt = p0 + lane < p1 ? im.pts[p0 + lane] : make_float2(0.0f, 0.0f);
        for (int p = p0 + lane; p < p1; p += 32) {
            const float2 xy = nxt;
            if (p + 32 < p1)
                nxt = im.pts[p + 32];
#pragma unroll
            for (int k = 0; k < NK; k++) {
                const int j = conv_bits<CV>(rho_f<UNIT>(xy.x, xy.y, c[k], sn[k], irho)) - base;
                red_smem(kb[k] + min((unsigned)j, (unsigned)nj) * 4u);
            }
        }
    }
}

template <bool UNIT, int NK>
__device__ __forceinline__ void window_tiles_cv(int cv, const hl_vote_img &im,
                                                const unsigned short *hits, int nhit,
                                                const float *s_c, const float *s_s, int base,
                                                int nj, unsigned acc_base, float irho)
{
    if (cv == CV_FLOOR)
        window_tiles_nk<UNIT, CV_FLOOR, NK>(im, hits, nhit, s_c, s_s, base, nj, acc_base, irho);
    else if (cv == CV_CEIL)
        window_tiles_nk<UNIT, CV_CEIL, NK>(im, hits, nhit, s_c, s_s, base, nj, acc_base, irho);
    else
        window_tiles_nk<UNIT, CV_EXACT, NK>(im, hits, nhit, s_c, s_s, base, nj, acc_base, irho);
}

/* windows with more thetas than the shared table: the same walk, cos/sin
 * from global memory, exact conversion */
template <bool UNIT>
__device__ __noinline__ void window_tiles_wide(const hl_vote_img &im, const unsigned *tmask,
                                               int ntl, const unsigned short *hits, int nhit,
                                               const float *c, const float *s, int nk,
                                               int base, int nj, unsigned acc_base, float irho)
{
    window_tiles<UNIT, CV_EXACT>(im, tmask, ntl, hits, nhit, c, s, nk, base, nj, acc_base,
                                 irho);
}

/* five CTAs an SM (48 registers): the vote waits on point loads, and more
 * resident warps hide them (uneven 512-4096 scenes without fall-back: +11%
 * against four CTAs; 2048 x 2048 scenes within 1.5%) */
template <bool UNIT>
__global__ void __launch_bounds__(256, 5)
hl_window_vote_kernel(hl_window_args a)
{
    extern __shared__ int wacc[];            /* [nk][nj + 1] haloed window, dump row nj */
    __shared__ unsigned tmask[HL_WIN_MAXTILES / 32];
    __shared__ float s_c[HL_WIN_MAXK], s_s[HL_WIN_MAXK];   /* its cos / sin */
    __shared__ unsigned short s_hit[HL_WIN_HITS];           /* its hit tiles */
    __shared__ int s_nhit;
    __shared__ int4 cur;
    const unsigned acc_base = (unsigned)__cvta_generic_to_shared(wacc);
    const int nwin = min(*a.nwin, a.cap);
    for (int wi = blockIdx.x; wi < nwin; wi += gridDim.x) {
        __syncthreads();
        if (threadIdx.x == 0)
            cur = a.win[wi];
        __syncthreads();
        const int b = cur.x, t = cur.y, r = cur.z, r1 = cur.w;   /* rho cells r .. r1 */
        const hl_vote_img im = a.vimgs[b];
        const hl_peak_img pk = a.pimgs[b];
        int k_lo, k_hi, j_lo, j_hi, unused;
        fine_range(t, HL_COARSE_T, a.T, &k_lo, &k_hi);
        fine_range(r, HL_COARSE_R, im.R, &j_lo, &unused);
        fine_range(r1, HL_COARSE_R, im.R, &unused, &j_hi);
        if (k_hi <= k_lo || j_hi <= j_lo)
            continue;
        /* haloed ranges, clipped to the accumulator */
        const int hk0 = max(k_lo - 1, 0), hk1 = min(k_hi + 1, a.T);
        const int hj0 = max(j_lo - 1, 0), hj1 = min(j_hi + 1, im.R);
        const int nk = hk1 - hk0, nj = hj1 - hj0;
        for (int i = threadIdx.x; i < nk * (nj + 1); i += blockDim.x)
            wacc[i] = 0;
        for (int i = threadIdx.x; i < HL_WIN_MAXK; i += blockDim.x) {
            s_c[i] = i < nk ? a.cosv[hk0 + i] : 0.0f;   /* past nk: a column nothing reads */
            s_s[i] = i < nk ? a.sinv[hk0 + i] : 0.0f;
        }
        /* tile filter over the image's tiles (one bit each) */
        const float c0 = a.cosv[hk0], s0 = a.sinv[hk0];
        const float c1 = a.cosv[hk1 - 1], s1 = a.sinv[hk1 - 1];
        const float lo_bin = (float)(im.rho_min + hj0);
        const float hi_bin = (float)(im.rho_min + hj1 - 1);
        const int ntl = min(im.ntiles, HL_WIN_MAXTILES);
        for (int base = 0; base < ntl; base += blockDim.x) {
            const int tl = base + threadIdx.x;
            const bool hit = tl < ntl && tile_hits(tl, im.tiles_x, im.w, im.h, c0, s0,
                                                   c1, s1, lo_bin, hi_bin, a.irho);
            const unsigned m = __ballot_sync(FULL, hit);
            if ((threadIdx.x & 31) == 0 && base + threadIdx.x < HL_WIN_MAXTILES)
                tmask[(base + threadIdx.x) >> 5] = m;
        }
        __syncthreads();
        /* the hit tiles listed in order (warp 0: a word per lane, prefix of
         * the counts, each lane writes its word's tiles) */
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x, nwd = (ntl + 31) / 32;
            int tot = 0;
            for (int w0 = 0; w0 < nwd; w0 += 32) {
                unsigned m = w0 + lane < nwd ? tmask[w0 + lane] : 0u;
                const int cnt = __popc(m);
                int incl = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o)
                        incl += t;
                }
                int pos = tot + incl - cnt;
                while (m) {
                    const int bb = __ffs(m) - 1;
                    m &= m - 1;
                    if (pos < HL_WIN_HITS)
                        s_hit[pos] = (unsigned short)((w0 + lane) * 32 + bb);
                    pos++;
                }
                tot += __shfl_sync(FULL, incl, 31);
            }
            if (lane == 0)
                s_nhit = tot;
        }
        __syncthreads();
        /* vote: each warp takes hit tiles in turn, its lanes the tile's
         * points; the float -> integer step by the magic constant unless the
         * window holds rho 0 (or has more thetas than the table) */
        {
            const int row_lo = im.rho_min + hj0, row_hi = im.rho_min + hj1 - 1;
            const int cv = row_lo >= 1 ? CV_FLOOR : (row_hi <= -1 ? CV_CEIL : CV_EXACT);
            const int base = cv == CV_EXACT ? row_lo : RHO_MAGIC_BITS + row_lo;
            if (s_nhit <= HL_WIN_HITS && nk <= 6 && a.nk_fast == 6)
                window_tiles_cv<UNIT, 6>(cv, im, s_hit, s_nhit, s_c, s_s, base, nj, acc_base,
                                         a.irho);
            else if (s_nhit <= HL_WIN_HITS && nk <= 10 && a.nk_fast == 10)
                window_tiles_cv<UNIT, 10>(cv, im, s_hit, s_nhit, s_c, s_s, base, nj, acc_base,
                                          a.irho);
            else if (nk <= HL_WIN_MAXK && row_lo >= 1)
                window_tiles<UNIT, CV_FLOOR>(im, tmask, ntl, s_hit, s_nhit, s_c, s_s, nk,
                                             RHO_MAGIC_BITS + row_lo, nj, acc_base, a.irho);
            else if (nk <= HL_WIN_MAXK && row_hi <= -1)
                window_tiles<UNIT, CV_CEIL>(im, tmask, ntl, s_hit, s_nhit, s_c, s_s, nk,
                                            RHO_MAGIC_BITS + row_lo, nj, acc_base, a.irho);
            else if (nk <= HL_WIN_MAXK)
                window_tiles<UNIT, CV_EXACT>(im, tmask, ntl, s_hit, s_nhit, s_c, s_s, nk,
                                             row_lo, nj, acc_base, a.irho);
            else
                window_tiles_wide<UNIT>(im, tmask, ntl, s_hit, s_nhit, a.cosv + hk0,
                                        a.sinv + hk0, nk, row_lo, nj, acc_base, a.irho);
        }
        __syncthreads();
        /* peaks among the owned bins */
        const int ok = k_hi - k_lo, oj = j_hi - j_lo;
        for (int i = threadIdx.x; i < ok * oj; i += blockDim.x) {
            const int k = k_lo + i / oj, j = j_lo + i % oj;
            const int lk = k - hk0, lj = j - hj0;
            const int v = wacc[lk * (nj + 1) + lj];
            bool is = false;
            if (v > pk.threshold) {
                const int W = (k > 0) ? wacc[(lk - 1) * (nj + 1) + lj] : 0;
                const int E = (k + 1 < a.T) ? wacc[(lk + 1) * (nj + 1) + lj] : 0;
                const int N = (j > 0) ? wacc[lk * (nj + 1) + lj - 1] : 0;
                const int S = (j + 1 < im.R) ? wacc[lk * (nj + 1) + lj + 1] : 0;
                /* okano_3_0/HoughLine.cu:195-199 */
                is = v > W && v >= E && v > N && v >= S;
            }
            if (is) {
                const unsigned idx = (unsigned)j * (unsigned)a.T + (unsigned)k;
                const unsigned long long key =
                    ((unsigned long long)(unsigned)v << 32) | (unsigned)(~idx);
                const int pos = atomicAdd(pk.ncand, 1);
                if (pos < pk.cap)
                    pk.keys[pos] = key;
                else
                    atomicOr(a.status, HL_ST_CAND_OVERFLOW);
            }
        }
        if (a.votes && threadIdx.x == 0) {
            /* executed votes: every point of every hit tile times the thetas */
            long long n = 0;
            for (int wd = 0; wd < (ntl + 31) / 32; wd++) {
                unsigned m = tmask[wd];
                while (m) {
                    const int tl = wd * 32 + __ffs(m) - 1;
                    m &= m - 1;
                    n += im.tile_off[tl + 1] - im.tile_off[tl];
                }
            }
            atomicAdd(a.votes, (unsigned long long)(n * nk));
        }
    }
}

template <bool UNIT>
static cudaError_t launch_window_t(const hl_window_args *a, size_t smem, int grid, cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(hl_window_vote_kernel<UNIT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    /* the CTAs take windows grid-stride: as many as are resident at once */
    int dev = 0, sms = 1, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hl_window_vote_kernel<UNIT>, 256,
                                                      smem) == cudaSuccess &&
        per_sm > 0)
        grid = std::min(grid, per_sm * sms);
    hl_window_vote_kernel<UNIT><<<grid, 256, smem, s>>>(*a);
    return cudaGetLastError();
}

cudaError_t hl_launch_window_vote(const hl_window_args *a, int max_win_bins, int grid,
                                  cudaStream_t s)
{
    const size_t smem = sizeof(int) * (size_t)max_win_bins;
    return a->irho == 1.0f ? launch_window_t<true>(a, smem, grid, s)
                           : launch_window_t<false>(a, smem, grid, s);
}
