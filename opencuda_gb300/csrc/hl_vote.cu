/*
 * hl_vote.cu -- stage (b): (theta, rho) int32 voting.
 *
 * Vote rule (okano_3_0/HoughLine.cu:86-130): an edge point (x, y) adds one
 * to bin (k, trunc(fl(x*cos_k) + fl(y*sin_k))) for every k.  The products and
 * the sum are rounded separately (__fmul_rn / __fadd_rn: no FMA contraction),
 * the float is truncated toward zero (the reference's +-0.5 step after the
 * (int) cast is a no-op), and cos_k/sin_k come from the GPU-evaluated table.
 *
 * Work decomposition.  A work item is one (theta slice, rho window) block of
 * the accumulator, held in shared memory as acc[row][lane]: 32 thetas (one
 * per lane) x win_rows rho bins.  A warp votes one point at a time; its 32
 * lanes add to 32 different thetas of the same point -- 32 different banks --
 * so every shared-memory reduction is conflict-free and no two lanes ever hit
 * one address (the aggregation a warp-aggregated atomic would buy is built
 * into the layout).
 *
 * Pipeline.  Persistent CTAs take items heaviest-first from a global counter.
 * For an item, all threads mark the 128x32 compaction tiles whose rho
 * interval over the slice meets the window and turn the marks into runs of
 * tiles -- contiguous ranges of the tile-major point list, 16-byte aligned
 * because the compaction pads every tile to an even number of float2
 * entries.  The runs, laid end to end, form the item's point stream.  Then
 * the CTA splits into one producer warp and consumer warps that meet only on
 * mbarriers: a batch is 64 points per consumer warp, batch b the stream
 * range [b*B, (b+1)*B); the producer's lanes each copy one run's part of it
 * into a ring of HL_VOTE_SLOTS shared-memory slots with cp.async.bulk (TMA
 * bulk copies completing on the slot's full barrier), so a slot holds its
 * batch gap-free; consumer warp i votes points [64i, 64i + 64) of the slot
 * straight from shared memory and arrives on the slot's empty barrier, which
 * the producer waits on before refilling it.  No block-wide barrier
 * separates batches.
 * At the end of the item the block is stored with coalesced 128-byte rows
 * into acc[R][Tp]; every bin is written exactly once, so the global
 * accumulator needs no clearing.
 *
 * Per point and consumer warp: half a broadcast shared load (16-byte loads
 * of point pairs), two multiplies, two adds (the second one rounds to an
 * integer, see vote_row), one subtract, one unsigned min, one address
 * multiply-add and one red.shared -- under nine issue slots and no branch
 * per vote.
 *
 * Bounds: every vote's row is clamped to the window's dump row (lanes past
 * the last theta to row 0 of their padding column, zeroed before the store),
 * mbarrier waits are bounded (a time-out sets a status bit that the host
 * reads with the result; every warp still reaches the same block barriers).
 */
#include "hl_internal.h"
#include "hl_device.cuh"

#define FULL 0xffffffffu
#define MBAR_WAIT_LIMIT (1 << 14)
/* float2 entries of one ring slot (runs are gap-free: the compaction pads
 * every tile to an even number of points, 16 bytes) */
#define SLOT_CAP HL_VOTE_CHUNK

/* Float -> integer without the conversion pipe (16 results per SM-clock).
 * M = 1.5 * 2^23: for |v| < 2^22 the sum v + M lies in [2^23, 2^24), where
 * floats are spaced 1 apart, so the sum rounded toward zero is M + floor(v)
 * and rounded up is M + ceil(v), and its bit pattern is bits(M) plus that
 * integer.  Truncation equals floor for v >= 0 and ceil for v < 0, so a rho
 * window whose rows are all >= 1 may use floor (a negative v then lands below
 * the window either way), one whose rows are all <= -1 may use ceil, and only
 * the window holding row 0 needs the exact conversion. */
#define RHO_MAGIC 12582912.0f
#define RHO_MAGIC_BITS 0x4B400000
enum { CV_EXACT = 0, CV_FLOOR = 1, CV_CEIL = 2 };

/* window-relative row of a point for this lane's theta; base is the rho of
 * row 0 (CV_EXACT) or RHO_MAGIC_BITS plus that rho */
template <bool UNIT, int CV>
__device__ __forceinline__ unsigned vote_row(float x, float y, float c,
                                             float s, float irho, int base)
{
    const float v = rho_f<UNIT>(x, y, c, s, irho);
    int r;
    if (CV == CV_FLOOR)
        r = __float_as_int(__fadd_rz(v, RHO_MAGIC));
    else if (CV == CV_CEIL)
        r = __float_as_int(__fadd_ru(v, RHO_MAGIC));
    else
        r = __float2int_rz(v);
    return (unsigned)(r - base);
}

/* ---- mbarrier + bulk copy ---------------------------------------------- */
__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned n)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(n)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar,
                                               unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                     smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src,
                                         unsigned bytes,
                                         unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
/* bounded wait for the phase with the given parity (false on time-out);
 * each try_wait may suspend the warp for up to about a microsecond instead
 * of spinning, leaving issue slots to working warps */
__device__ __forceinline__ bool mbar_wait_sleep(unsigned long long *bar,
                                                unsigned parity)
{
    const unsigned a = smem_u32(bar);
    for (int i = 0; i < MBAR_WAIT_LIMIT; i++) {
        unsigned ok;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], "
            "%2, %3; selp.u32 %0, 1, 0, p; }"
            : "=r"(ok)
            : "r"(a), "r"(parity), "r"(1000u)
            : "memory");
        if (ok)
            return true;
    }
    return false;
}

/* 32 points (16 float4 pairs) of one consumer warp's share, no bounds */
template <bool UNIT, int CV>
__device__ __forceinline__ void vote_share32(const float2 *pts, float c,
                                             float s, float irho, int base,
                                             unsigned acc_l, unsigned lim);

/* one vote, no returned value */
__device__ __forceinline__ void red_smem(unsigned addr)
{
    asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(addr));
}

/* Votes of a consumer warp for points j, j + step, ... < n of a ring slot.
 * A row outside the window (rl >= lim as unsigned) is sent to row lim: the
 * dump row just past the window (lim = window rows) or, for lanes past the
 * last theta (lim = 0), row 0 of the lane's own padding column.  No vote is
 * predicated, so the loop has no branch per vote. */
template <bool UNIT, int CV>
__device__ __forceinline__ void vote_batch(const float2 *pts, int n, int j,
                                           int step, float c, float s,
                                           float irho, int base,
                                           unsigned acc_l, unsigned lim)
{
    for (; j + 3 * step < n; j += 4 * step) {
        const float2 p0 = pts[j];
        const float2 p1 = pts[j + step];
        const float2 p2 = pts[j + 2 * step];
        const float2 p3 = pts[j + 3 * step];
        const unsigned l0 = min(vote_row<UNIT, CV>(p0.x, p0.y, c, s, irho, base), lim);
        const unsigned l1 = min(vote_row<UNIT, CV>(p1.x, p1.y, c, s, irho, base), lim);
        const unsigned l2 = min(vote_row<UNIT, CV>(p2.x, p2.y, c, s, irho, base), lim);
        const unsigned l3 = min(vote_row<UNIT, CV>(p3.x, p3.y, c, s, irho, base), lim);
        red_smem(acc_l + 128u * l0);
        red_smem(acc_l + 128u * l1);
        red_smem(acc_l + 128u * l2);
        red_smem(acc_l + 128u * l3);
    }
    for (; j < n; j += step) {
        const float2 p0 = pts[j];
        red_smem(acc_l + 128u * min(vote_row<UNIT, CV>(p0.x, p0.y, c, s, irho, base), lim));
    }
}

template <bool UNIT, int CV>
__device__ __forceinline__ void vote_share32(const float2 *pts, float c,
                                             float s, float irho, int base,
                                             unsigned acc_l, unsigned lim)
{
    const float4 *q = reinterpret_cast<const float4 *>(pts);
#pragma unroll
    for (int i = 0; i < 16; i += 2) {
        const float4 u = q[i], w = q[i + 1];
        const unsigned l0 = min(vote_row<UNIT, CV>(u.x, u.y, c, s, irho, base), lim);
        const unsigned l1 = min(vote_row<UNIT, CV>(u.z, u.w, c, s, irho, base), lim);
        const unsigned l2 = min(vote_row<UNIT, CV>(w.x, w.y, c, s, irho, base), lim);
        const unsigned l3 = min(vote_row<UNIT, CV>(w.z, w.w, c, s, irho, base), lim);
        red_smem(acc_l + 128u * l0);
        red_smem(acc_l + 128u * l1);
        red_smem(acc_l + 128u * l2);
        red_smem(acc_l + 128u * l3);
    }
}

/* a consumer warp's share of a slot: up to 32 points starting at pts */
template <bool UNIT, int CV>
__device__ __forceinline__ void vote_share(const float2 *pts, int m, float c,
                                           float s, float irho, int base,
                                           unsigned acc_l, unsigned lim)
{
    if (m >= 32)
        vote_share32<UNIT, CV>(pts, c, s, irho, base, acc_l, lim);
    else if (m > 0)
        vote_batch<UNIT, CV>(pts, m, 0, 1, c, s, irho, base, acc_l, lim);
}

struct VoteSmem {
    hl_vote_img im;                    /* the current item's image */
    unsigned long long full[HL_VOTE_SLOTS];
    unsigned long long empty[HL_VOTE_SLOTS];
    int item;
    int part;
    int nruns;
    int timeout;
    int total;                         /* points in the group's runs */
    unsigned mask[HL_VOTE_TG / 32];
    unsigned sw[HL_VOTE_TG / 32];      /* run starts per mask word */
    unsigned ew[HL_VOTE_TG / 32];      /* run ends per mask word */
    int ws[HL_VOTE_TG / 32];           /* runs starting before the word */
    int we[HL_VOTE_TG / 32];
    int run_s[HL_VOTE_TG / 2];
    int run_e[HL_VOTE_TG / 2];
    int rpre[HL_VOTE_TG / 2];          /* stream position of each run */
    alignas(16) float2 raw[HL_VOTE_SLOTS][SLOT_CAP];
};

#define VOTE_FIXED ((sizeof(VoteSmem) + 127) / 128 * 128)

/* the window's rows plus the dump row */
size_t hl_vote_smem_bytes(int win_rows)
{
    return VOTE_FIXED + (size_t)(win_rows + 1) * HL_SLICE * sizeof(int);
}

int hl_vote_max_rows(void)
{
    const size_t cap = 227u * 1024u;
    return (int)((cap - VOTE_FIXED) / (HL_SLICE * sizeof(int)) - 1) & ~7;
}

template <bool UNIT>
__global__ void __launch_bounds__(1024, 1)
hl_vote_kernel(hl_vote_args a)
{
    extern __shared__ __align__(128) unsigned char vote_raw[];
    VoteSmem &sm = *reinterpret_cast<VoteSmem *>(vote_raw);
    int *s_acc = reinterpret_cast<int *>(vote_raw + VOTE_FIXED);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nthr = blockDim.x, nwarps = nthr >> 5;
    const int ncons = nwarps - 1;               /* consumer warps 1..nwarps-1 */
    /* points per batch: 64 per consumer warp (at most SLOT_CAP) */
    const int batch = 64 * ncons;
    const int nslices = a.Tp / HL_SLICE;

    if (tid == 0) {
        for (int i = 0; i < HL_VOTE_SLOTS; i++) {
            mbar_init(&sm.full[i], 1);
            mbar_init(&sm.empty[i], (unsigned)ncons);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sm.timeout = 0;
    }
    /* running batch index, the same sequence on the producer and consumers:
     * slot = seq % SLOTS, phase = (seq / SLOTS) & 1 */
    unsigned seq = 0;
    __syncthreads();

    while (true) {
        if (tid == 0) {
            const unsigned t = atomicAdd(a.work, 1u) - a.work_base;
            if (t < (unsigned)a.nitems) {
                const int2 it = a.items[t];
                sm.item = it.x & 0xffff;
                sm.part = it.y;
                sm.im = a.imgs ? a.imgs[(unsigned)it.x >> 16] : a.img0;
            } else {
                sm.item = -1;
            }
        }
        __syncthreads();
        const int item = sm.item;
        if (item < 0)
            break;
        const int part = sm.part & 0xffff, nparts = max(sm.part >> 16, 1);
        const int slice = item % nslices, win = item / nslices;
        const int k0 = slice * HL_SLICE, k = k0 + lane;
        const float c = a.cosv[k], s = a.sinv[k];   /* table padded to Tp */
        const int w0 = win * a.win_rows;
        const int rows = min(a.win_rows, sm.im.R - w0);
        const int row_base = sm.im.rho_min + w0;   /* rho bin of local row 0 */
        const unsigned lrows = (k < a.T) ? (unsigned)rows : 0u;
        const int cv = row_base >= 1 ? CV_FLOOR
                       : (row_base + rows - 1 <= -1 ? CV_CEIL : CV_EXACT);
        const int vbase = cv == CV_EXACT ? row_base : RHO_MAGIC_BITS + row_base;
        const int klast = min(k0 + HL_SLICE - 1, a.T - 1);
        const float c0 = a.cosv[k0], s0 = a.sinv[k0];
        const float c1 = a.cosv[klast], s1 = a.sinv[klast];
        const float lo_bin = (float)row_base;
        const float hi_bin = (float)(row_base + rows - 1);
        const bool filter = sm.im.nwin > 1;
        const int ntiles = sm.im.ntiles, tiles_x = sm.im.tiles_x;
        const int img_w = sm.im.w, img_h = sm.im.h;
        const int *tile_off = sm.im.tile_off;
        const float2 *pts_g = sm.im.pts;
        int32_t *acc_g = sm.im.acc;
        const unsigned acc_l = smem_u32(s_acc) + 4u * lane;

        {
            int4 *z = reinterpret_cast<int4 *>(s_acc);
            const int4 zero = make_int4(0, 0, 0, 0);
            for (int i = tid; i < rows * (HL_SLICE / 4); i += nthr)
                z[i] = zero;
        }

        for (int tg = 0; tg < ntiles; tg += HL_VOTE_TG) {
            const int tg_n = min(HL_VOTE_TG, ntiles - tg);
            /* coarse filter: one bit per tile of the group */
            for (int wd = warp; wd < HL_VOTE_TG / 32; wd += nwarps) {
                const int tl = wd * 32 + lane;
                bool hit = false;
                if (tl < tg_n)
                    hit = !filter || tile_hits(tg + tl, tiles_x, img_w, img_h, c0,
                                               s0, c1, s1, lo_bin, hi_bin,
                                               a.irho);
                const unsigned m = __ballot_sync(FULL, hit);
                if (lane == 0)
                    sm.mask[wd] = m;
            }
            __syncthreads();
            /* run boundaries per word and their prefix counts (warp 0, four
             * words per lane) */
            if (warp == 0) {
                constexpr int WPL = HL_VOTE_TG / 32 / 32;
                int cs = 0, ce = 0;
                unsigned st[WPL], en[WPL];
#pragma unroll
                for (int q = 0; q < WPL; q++) {
                    const int wd = lane * WPL + q;
                    const unsigned m = sm.mask[wd];
                    const unsigned prev = (wd > 0) ? sm.mask[wd - 1] : 0u;
                    const unsigned next = (wd + 1 < HL_VOTE_TG / 32) ? sm.mask[wd + 1] : 0u;
                    st[q] = m & ~((m << 1) | (prev >> 31));
                    en[q] = m & ~((m >> 1) | ((next & 1u) << 31));
                    cs += __popc(st[q]);
                    ce += __popc(en[q]);
                }
                int is = cs, ie = ce;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t1 = __shfl_up_sync(FULL, is, o);
                    const int t2 = __shfl_up_sync(FULL, ie, o);
                    if (lane >= o) {
                        is += t1;
                        ie += t2;
                    }
                }
                is -= cs;
                ie -= ce;
#pragma unroll
                for (int q = 0; q < WPL; q++) {
                    const int wd = lane * WPL + q;
                    sm.sw[wd] = st[q];
                    sm.ew[wd] = en[q];
                    sm.ws[wd] = is;
                    sm.we[wd] = ie;
                    is += __popc(st[q]);
                    ie += __popc(en[q]);
                }
                if (lane == 31)
                    sm.nruns = is;
            }
            __syncthreads();
            /* run endpoints -> point ranges, one tile per thread */
            for (int tl = tid; tl < tg_n; tl += nthr) {
                const int wd = tl >> 5, b = tl & 31;
                const unsigned below = (1u << b) - 1u;
                if ((sm.sw[wd] >> b) & 1u)
                    sm.run_s[sm.ws[wd] + __popc(sm.sw[wd] & below)] = tile_off[tg + tl];
                if ((sm.ew[wd] >> b) & 1u)
                    sm.run_e[sm.we[wd] + __popc(sm.ew[wd] & below)] = tile_off[tg + tl + 1];
            }
            __syncthreads();

            /* stream positions of the runs (warp 0: a chunk of runs per
             * lane, then a warp scan of the chunk sums) */
            if (warp == 0) {
                const int nr = sm.nruns;
                const int per = (nr + 31) / 32;
                const int r0 = min(nr, lane * per), r1 = min(nr, r0 + per);
                int sum = 0;
                for (int r = r0; r < r1; r++)
                    sum += sm.run_e[r] - sm.run_s[r];
                int incl = sum;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o)
                        incl += t;
                }
                int pos = incl - sum;
                for (int r = r0; r < r1; r++) {
                    sm.rpre[r] = pos;
                    pos += sm.run_e[r] - sm.run_s[r];
                }
                if (lane == 31)
                    sm.total = incl;
            }
            __syncthreads();
            const int total = sm.total;
            const int nb_all = (total + batch - 1) / batch;
            /* this part's share of the batches */
            const int b_lo = (int)((long long)nb_all * part / nparts);
            const int b_hi = (int)((long long)nb_all * (part + 1) / nparts);
            const int nruns = sm.nruns;

            if (warp == 0) {
                /* producer warp: batch b is stream range [b*CHUNK, ...);
                 * lane i copies the part of run r0 + i overlapping it, and a
                 * ballot finds the first run of the next batch */
                int r0 = 0;
                {
                    /* first run ending after this part's first point */
                    const int s_first = b_lo * batch;
                    int lo = 0, hi = max(nruns - 1, 0);
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (sm.rpre[mid] + (sm.run_e[mid] - sm.run_s[mid]) <= s_first)
                            lo = mid + 1;
                        else
                            hi = mid;
                    }
                    r0 = lo;
                }
                for (int b = b_lo; b < b_hi; b++) {
                    const int slot = (int)(seq % HL_VOTE_SLOTS);
                    if (lane == 0 && seq >= HL_VOTE_SLOTS && !*(volatile int *)&sm.timeout &&
                        !mbar_wait_sleep(&sm.empty[slot], ((seq / HL_VOTE_SLOTS) - 1u) & 1u)) {
                        sm.timeout = 1;
                        atomicOr(a.status, HL_ST_VOTE_TIMEOUT);
                    }
                    const int s0 = b * batch;
                    const int e0 = min(total, s0 + batch);
                    if (lane == 0)
                        mbar_expect_tx(&sm.full[slot], (unsigned)(e0 - s0) * 8u);
                    __syncwarp();
                    /* runs from r0 on: every run ending at or before e0 lies
                     * wholly in this batch; the first one reaching past e0
                     * is shared with the next batch and ends the scan (the
                     * runs after it start at or beyond e0) */
                    int next = nruns;
                    for (int rb = r0; rb < nruns; rb += 32) {
                        const int r = rb + lane;
                        bool past = false;
                        if (r < nruns) {
                            const int rs = sm.rpre[r];
                            const int re = rs + (sm.run_e[r] - sm.run_s[r]);
                            const int ps = max(s0, rs), pe = min(e0, re);
                            if (pe > ps)
                                bulk_g2s(&sm.raw[slot][ps - s0],
                                         pts_g + sm.run_s[r] + (ps - rs),
                                         (unsigned)(pe - ps) * 8u, &sm.full[slot]);
                            past = re > e0;
                        }
                        const unsigned pm = __ballot_sync(FULL, past);
                        if (pm) {
                            next = rb + __ffs(pm) - 1;
                            break;
                        }
                    }
                    r0 = next;
                    seq++;
                }
            } else {
                /* consumer warps: vote every point of a batch, then free
                 * the slot */
                const int cw = warp - 1;
                for (int b = b_lo; b < b_hi; b++) {
                    const int slot = (int)(seq % HL_VOTE_SLOTS);
                    /* after a time-out nobody waits any more */
                    const bool ok = *(volatile int *)&sm.timeout ||
                                    mbar_wait_sleep(&sm.full[slot], (seq / HL_VOTE_SLOTS) & 1u);
                    if (!ok && lane == 0) {
                        sm.timeout = 1;
                        atomicOr(a.status, HL_ST_VOTE_TIMEOUT);
                    }
                    seq++;
                    /* this warp's share: points [64 cw, 64 cw + 64), two
                     * 32-point halves */
                    const int m = min(64, total - b * batch - 64 * cw);
                    const float2 *pts = sm.raw[slot] + 64 * cw;
                    if (cv == CV_FLOOR) {
                        vote_share<UNIT, CV_FLOOR>(pts, m, c, s, a.irho, vbase, acc_l, lrows);
                        vote_share<UNIT, CV_FLOOR>(pts + 32, m - 32, c, s, a.irho, vbase, acc_l, lrows);
                    } else if (cv == CV_CEIL) {
                        vote_share<UNIT, CV_CEIL>(pts, m, c, s, a.irho, vbase, acc_l, lrows);
                        vote_share<UNIT, CV_CEIL>(pts + 32, m - 32, c, s, a.irho, vbase, acc_l, lrows);
                    } else {
                        vote_share<UNIT, CV_EXACT>(pts, m, c, s, a.irho, vbase, acc_l, lrows);
                        vote_share<UNIT, CV_EXACT>(pts + 32, m - 32, c, s, a.irho, vbase, acc_l, lrows);
                    }
                    __syncwarp();
                    if (lane == 0)
                        mbar_arrive(&sm.empty[slot]);
                }
            }
            __syncthreads();
        }

        /* store the block: row i of the window -> acc[(w0 + i) * Tp + k0 ..] */
        int4 *dst4 = reinterpret_cast<int4 *>(acc_g);
        const int4 *src4 = reinterpret_cast<const int4 *>(s_acc);
        const int tp4 = a.Tp >> 2;
        /* row 0 of the padding columns (thetas >= T) holds dumped votes */
        if (nparts == 1) {
            for (int i = tid; i < rows * (HL_SLICE / 4); i += nthr) {
                const int rr = i >> 3, q = i & 7;
                int4 v = src4[i];
                if (rr == 0) {
                    const int kq = k0 + 4 * q;
                    if (kq >= a.T) v.x = 0;
                    if (kq + 1 >= a.T) v.y = 0;
                    if (kq + 2 >= a.T) v.z = 0;
                    if (kq + 3 >= a.T) v.w = 0;
                }
                dst4[(size_t)(w0 + rr) * tp4 + (k0 >> 2) + q] = v;
            }
        } else {
            /* one part of a split block: add its nonzero counts into the
             * zeroed accumulator */
            for (int i = tid; i < rows * HL_SLICE; i += nthr) {
                const int v = s_acc[i];
                if (v && k0 + (i & 31) < a.T)
                    atomicAdd(&acc_g[(size_t)(w0 + (i >> 5)) * a.Tp + k0 + (i & 31)], v);
            }
        }
        __syncthreads();
        if (sm.timeout)
            break;
    }
}

cudaError_t hl_launch_vote(const hl_vote_args *a, int threads, int grid,
                           cudaStream_t s)
{
    const size_t smem = hl_vote_smem_bytes(a->win_rows);
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

size_t hl_vote_points_smem_bytes(int win_rows)
{
    return (size_t)win_rows * HL_SLICE * sizeof(int);
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
    extern __shared__ __align__(16) int s_pacc[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    const int k0 = blockIdx.x * HL_SLICE, k = k0 + lane;
    const bool kvalid = k < T;
    const float c = cosv[k], s = sinv[k];
    const int w0 = blockIdx.y * win_rows;
    const int rows = min(win_rows, R - w0);
    const int row_base = rho_min + w0;
    for (int i = tid; i < rows * HL_SLICE; i += blockDim.x)
        s_pacc[i] = 0;
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
                atomicAdd(&s_pacc[row * HL_SLICE + lane], 1);
        }
    }
    __syncthreads();
    int4 *dst4 = reinterpret_cast<int4 *>(acc);
    const int4 *src4 = reinterpret_cast<const int4 *>(s_pacc);
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
    size_t smem = hl_vote_points_smem_bytes(win_rows);
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
