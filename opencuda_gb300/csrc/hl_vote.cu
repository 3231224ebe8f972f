/*
 * hl_vote.cu -- stage (b): (theta, rho) int32 voting.
 *
 * Vote rule (okano_3_0/HoughLine.cu:86-130): an edge point (x, y) adds one
 * to bin (k, trunc(fl(x*cos_k) + fl(y*sin_k))) for every k.  The products and
 * the sum are rounded separately (packed f32x2 products as fma(a, b, +0) and
 * a packed add: no FMA contraction, see f2_mul), the float is truncated
 * toward zero (the reference's +-0.5 step after the (int) cast is a no-op),
 * and cos_k/sin_k come from the GPU-evaluated table.
 *
 * Work decomposition.  A work item is one (theta slice, rho window) block of
 * the accumulator, held in shared memory as acc[row][column]: 32 thetas x
 * win_rows rho bins.  A warp votes 8 points at a time on the diagonal
 * schedule (DiagTab): at every step its 32 lanes add to 32 different theta
 * columns -- 32 different banks -- so every shared-memory reduction is
 * conflict-free and no two lanes ever hit one address (the aggregation a
 * warp-aggregated atomic would buy is built into the layout).
 *
 * Pipeline.  Persistent CTAs of one producer warp and consumer warps that
 * meet only on mbarriers.  The producer takes items heaviest-first from a
 * global counter.  For an item it reads the block's tile mask -- the 128x32
 * compaction tiles whose rho interval over the slice meets the window,
 * computed once per geometry by hl_tile_mask_kernel -- and turns it into
 * runs of tiles: contiguous ranges of the tile-major point list, 16-byte
 * aligned because the compaction pads every tile to an even number of
 * float2 entries.  The runs, laid end to end, form the item's point stream.
 * It publishes the item as a segment (double-buffered descriptor) and
 * streams it: a batch is HL_VOTE_PPW points per consumer warp, batch b the stream
 * range [b*B, (b+1)*B); the producer's lanes each copy one run's part of it
 * into a ring of HL_VOTE_SLOTS shared-memory slots with cp.async.bulk (TMA
 * bulk copies completing on the slot's full barrier), so a slot holds its
 * batch gap-free; consumer warp i votes points [PPW i, PPW i + PPW) of the slot
 * straight from shared memory and arrives on the slot's empty barrier, which
 * the producer waits on before refilling it.  The producer moves on to the
 * next item as soon as the current one is issued, so its setup and first
 * copies overlap the consumers' last batches.
 * When an item is voted the consumers store the block with coalesced
 * 128-byte rows into acc[R][Tp] (a part of a split block: into its scratch
 * slot, summed into the block by hl_merge_kernel) and clear it; every bin is
 * written exactly once, so the accumulator needs no clearing.
 *
 * Per vote: one packed multiply of x and one of y (two thetas per f32x2
 * instruction, so half of each), half a packed add, half a packed
 * magic-constant add (the float -> integer, see RHO_MAGIC), one clamp to the
 * dump row, one address add and one red.shared -- about five issue slots --
 * plus an eighth of a point load (the diagonal schedule, see DiagTab); no
 * branch per vote.
 *
 * Bounds: every vote's row is clamped to the window's dump row, one row past
 * the window in every column; the padding columns (thetas >= T) are stored
 * as zero.
 * After the start there is no block-wide barrier, and every mbarrier wait is
 * bounded: a time-out sets a status bit that the host reads with the result
 * and an abort flag on which every other waiting warp gives up too; the
 * producer then waits (bounded) for its copies in flight before exiting.
 */
#include "hl_internal.h"
#include "hl_device.cuh"

#define FULL 0xffffffffu
#define MBAR_WAIT_LIMIT (1 << 14)
/* float2 entries of one ring slot (runs are gap-free: the compaction pads
 * every tile to an even number of points, 16 bytes) */
#define SLOT_CAP HL_VOTE_CHUNK

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

/* A consumer warp's share of a slot: points [0, m) of pts, m <= HL_VOTE_PPW,
 * 8 per round.  Entries past m (stale ring data) vote as the sentinel
 * (1e30, 0), whose rows lie outside every window and go to the dump row. */
template <bool UNIT, int CV>
__device__ __forceinline__ void vote_share(const float2 *pts, int m, const DiagTab &t,
                                           f2x ir, int base, unsigned lim, int p)
{
    if (m >= HL_VOTE_PPW) {
#pragma unroll 2
        for (int r = 0; r < HL_VOTE_PPW; r += 8) {
            const float2 q = pts[r + p];
            diag_point<UNIT, CV>(q.x, q.y, t, ir, base, lim);
        }
    } else {
        for (int r = 0; r < m; r += 8) {
            float2 q = pts[r + p];
            if (r + p >= m)
                q = make_float2(1e30f, 0.0f);
            diag_point<UNIT, CV>(q.x, q.y, t, ir, base, lim);
        }
    }
}

/* Bounded wait that also gives up as soon as another warp of the CTA has
 * given up (*abort_flag set).  A time-out sets the flag and the status bit;
 * false means: leave the kernel. */
__device__ __forceinline__ bool mbar_wait_ab(unsigned long long *bar,
                                             unsigned parity, int *abort_flag,
                                             int *status)
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
        if (*(volatile int *)abort_flag)
            return false;
    }
    if ((threadIdx.x & 31) == 0)
        atomicOr(status, HL_ST_VOTE_TIMEOUT);
    *(volatile int *)abort_flag = 1;
    return false;
}

/* One segment of the producer's stream: one tile group (HL_VOTE_TG tiles)
 * of a work item, or the end of the work (item < 0). */
struct VoteSeg {
    int32_t *acc;                      /* the image's accumulator */
    int item;                          /* slice + nslices * window, or -1 */
    int part, nparts, slot;            /* see hl_vote_args.items */
    int rho_min, R;                    /* the image's rho range */
    int total;                         /* points in the segment's runs */
    int b_lo, b_hi;                    /* this part's batches of them */
    int first, last;                   /* first / last segment of the item */
    float c[HL_SLICE], s[HL_SLICE];    /* cos / sin of the slice's thetas */
    int img;                           /* the image (in the tail padding: the
                                          layout measured fastest is kept) */
};

struct VoteSmem {
    unsigned long long full[HL_VOTE_SLOTS];
    unsigned long long empty[HL_VOTE_SLOTS];
    unsigned long long seg_full[2];    /* producer -> consumers */
    unsigned long long seg_empty[2];   /* consumers -> producer */
    unsigned long long cbar;           /* barrier of the consumer threads */
    int abort;                         /* a warp gave up waiting */
    VoteSeg seg[2];
    int run_s[HL_VOTE_TG / 2];         /* producer: the segment's runs */
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

/* Admitted tiles of every (slice, window) block of an image: one warp per
 * mask word, lane = tile (tile_hits; every tile when the image has a single
 * window).  They depend on the geometry only, so callers compute them once
 * per geometry. */
__global__ void hl_tile_mask_kernel(hl_vote_args a)
{
    const hl_vote_img im = a.imgs ? a.imgs[blockIdx.y] : a.img0;
    const int words = (im.ntiles + 31) >> 5;
    const int nslices = a.Tp / HL_SLICE;
    const long long nw = (long long)nslices * im.nwin * words;
    const int lane = threadIdx.x & 31;
    const long long wstep = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long wd = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
         wd < nw; wd += wstep) {
        const int blk = (int)(wd / words), wi = (int)(wd % words);
        const int slice = blk % nslices, win = blk / nslices;
        const int k0 = slice * HL_SLICE;
        const int klast = min(k0 + HL_SLICE - 1, a.T - 1);
        const int w0 = win * a.win_rows;
        const int rows = min(a.win_rows, im.R - w0);
        const int t = wi * 32 + lane;
        bool hit = false;
        if (t < im.ntiles)
            hit = im.nwin <= 1 ||
                  tile_hits(t, im.tiles_x, im.w, im.h, a.cosv[k0], a.sinv[k0],
                            a.cosv[klast], a.sinv[klast],
                            (float)(im.rho_min + w0),
                            (float)(im.rho_min + w0 + rows - 1), a.irho);
        const unsigned m = __ballot_sync(FULL, hit);
        if (lane == 0)
            im.tmask[wd] = m;
    }
}

/* barrier of the consumer threads (every one arrives; bounded wait) */
__device__ __forceinline__ bool cons_sync(VoteSmem &sm, unsigned &par,
                                          int *status)
{
    mbar_arrive(&sm.cbar);
    const bool ok = mbar_wait_ab(&sm.cbar, par, &sm.abort, status);
    par ^= 1u;
    return ok;
}

/* Producer warp: takes items, turns each tile group of an item into a
 * segment (runs of admitted tiles -> point ranges -> batches), publishes the
 * segment and streams its batches into the ring.  It runs ahead of the
 * consumers by up to the ring's depth, so the next item's setup and first
 * copies overlap the current item's last votes. */
template <bool NOTE>
__device__ __forceinline__ void vote_producer(const hl_vote_args &a,
                                              VoteSmem &sm, int batch)
{
    const int lane = threadIdx.x & 31;
    const int nslices = a.Tp / HL_SLICE;
    unsigned seq = 0;    /* batches issued */
    unsigned nseg = 0;   /* segments published */
    bool ok = true;
    while (ok) {
        unsigned t = 0;
        if (lane == 0)
            t = atomicAdd(a.work, 1u) - a.work_base;
        t = __shfl_sync(FULL, t, 0);
        const bool have = t < (unsigned)a.nitems;
        int4 it = make_int4(-1, 0, 0, 0);
        hl_vote_img im = a.img0;
        if (have) {
            it = a.items[t];
            if (a.imgs)
                im = a.imgs[(unsigned)it.x >> 16];
        }
        const int item = have ? (it.x & 0xffff) : -1;
        const int part = it.y & 0xffff, nparts = max(it.y >> 16, 1);
        const int k0 = have ? (item % nslices) * HL_SLICE : 0;
        const float cl = have ? a.cosv[k0 + lane] : 0.0f;
        const float sl = have ? a.sinv[k0 + lane] : 0.0f;
        const int ntiles = have ? im.ntiles : 0;
        const int words = (ntiles + 31) >> 5;
        const unsigned *mk = have ? im.tmask + (size_t)item * words : nullptr;
        int tg = 0;
        do {
            const int tg_n = min(HL_VOTE_TG, ntiles - tg);
            int total = 0, nruns = 0;
            if (have) {
                /* runs of the group's mask words, four words per lane */
                constexpr int WPL = HL_VOTE_TG / 32 / 32;
                unsigned m[WPL], st[WPL], en[WPL];
                int cs = 0, ce = 0;
#pragma unroll
                for (int q = 0; q < WPL; q++) {
                    const int wd = lane * WPL + q;
                    m[q] = wd * 32 < tg_n ? mk[(tg >> 5) + wd] : 0u;
                }
                unsigned prev = __shfl_up_sync(FULL, m[WPL - 1], 1);
                unsigned next = __shfl_down_sync(FULL, m[0], 1);
                if (lane == 0)
                    prev = 0u;
                if (lane == 31)
                    next = 0u;
#pragma unroll
                for (int q = 0; q < WPL; q++) {
                    const unsigned pv = q > 0 ? m[q - 1] : prev;
                    const unsigned nx = q + 1 < WPL ? m[q + 1] : next;
                    st[q] = m[q] & ~((m[q] << 1) | (pv >> 31));
                    en[q] = m[q] & ~((m[q] >> 1) | ((nx & 1u) << 31));
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
                nruns = __shfl_sync(FULL, is, 31);
                is -= cs;
                ie -= ce;
                /* tile indices of the run ends, then their point offsets
                 * (four loads in flight per lane) */
#pragma unroll
                for (int q = 0; q < WPL; q++) {
                    const int base = (lane * WPL + q) * 32;
                    for (unsigned x = st[q]; x; x &= x - 1)
                        sm.run_s[is++] = base + __ffs(x) - 1;
                    for (unsigned x = en[q]; x; x &= x - 1)
                        sm.run_e[ie++] = base + __ffs(x);
                }
                __syncwarp();
                const int *toff = im.tile_off + tg;
                for (int r0 = 0; r0 < nruns; r0 += 128) {
                    int vs[4], ve[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int r = r0 + 32 * u + lane;
                        if (r < nruns) {
                            vs[u] = toff[sm.run_s[r]];
                            ve[u] = toff[sm.run_e[r]];
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int r = r0 + 32 * u + lane;
                        if (r < nruns) {
                            sm.run_s[r] = vs[u];
                            sm.run_e[r] = ve[u];
                        }
                    }
                }
                __syncwarp();
                /* stream positions: a chunk of runs per lane, warp scan */
                const int per = (nruns + 31) / 32;
                const int ra = min(nruns, lane * per), rb = min(nruns, ra + per);
                int sum = 0;
                for (int r = ra; r < rb; r++)
                    sum += sm.run_e[r] - sm.run_s[r];
                int incl = sum;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t1 = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o)
                        incl += t1;
                }
                int pos = incl - sum;
                for (int r = ra; r < rb; r++) {
                    sm.rpre[r] = pos;
                    pos += sm.run_e[r] - sm.run_s[r];
                }
                total = __shfl_sync(FULL, incl, 31);
                __syncwarp();
            }
            const int nb_all = (total + batch - 1) / batch;
            const int b_lo = (int)((long long)nb_all * part / nparts);
            const int b_hi = (int)((long long)nb_all * (part + 1) / nparts);

            /* publish the segment once the consumers are done with the one
             * that last used its slot */
            const int ds = (int)(nseg & 1u);
            if (nseg >= 2 &&
                !mbar_wait_ab(&sm.seg_empty[ds], ((nseg >> 1) - 1u) & 1u, &sm.abort,
                              a.status)) {
                ok = false;
                break;
            }
            VoteSeg &g = sm.seg[ds];
            g.c[lane] = cl;
            g.s[lane] = sl;
            if (lane == 0) {
                g.acc = im.acc;
                g.item = item;
                g.part = part;
                g.nparts = nparts;
                g.slot = it.z;
                if (NOTE)
                    g.img = a.imgs ? (int)((unsigned)it.x >> 16) : 0;
                g.rho_min = im.rho_min;
                g.R = im.R;
                g.total = total;
                g.b_lo = b_lo;
                g.b_hi = b_hi;
                g.first = tg == 0;
                g.last = tg + HL_VOTE_TG >= ntiles;
            }
            __syncwarp();
            if (lane == 0)
                mbar_arrive(&sm.seg_full[ds]);
            nseg++;
            if (!have)
                break;

            /* batch b is stream range [b * batch, ...): lane i copies the
             * part of run r0 + i overlapping it; a ballot finds the first run
             * of the next batch */
            int r0 = 0;
            {
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
            for (int b = b_lo; b < b_hi && ok; b++) {
                const int slot = (int)(seq % HL_VOTE_SLOTS);
                if (seq >= HL_VOTE_SLOTS &&
                    !mbar_wait_ab(&sm.empty[slot], ((seq / HL_VOTE_SLOTS) - 1u) & 1u,
                                  &sm.abort, a.status)) {
                    ok = false;
                    break;
                }
                const int s0 = b * batch;
                const int e0 = min(total, s0 + batch);
                if (lane == 0)
                    mbar_expect_tx(&sm.full[slot], (unsigned)(e0 - s0) * 8u);
                __syncwarp();
                /* runs from r0 on: every run ending at or before e0 lies
                 * wholly in this batch; the first one reaching past e0 is
                 * shared with the next batch and ends the scan */
                int nextr = nruns;
                for (int rb = r0; rb < nruns; rb += 32) {
                    const int r = rb + lane;
                    bool past = false;
                    if (r < nruns) {
                        const int rs = sm.rpre[r];
                        const int re = rs + (sm.run_e[r] - sm.run_s[r]);
                        const int ps = max(s0, rs), pe = min(e0, re);
                        if (pe > ps)
                            bulk_g2s(&sm.raw[slot][ps - s0], im.pts + sm.run_s[r] + (ps - rs),
                                     (unsigned)(pe - ps) * 8u, &sm.full[slot]);
                        past = re > e0;
                    }
                    const unsigned pm = __ballot_sync(FULL, past);
                    if (pm) {
                        nextr = rb + __ffs(pm) - 1;
                        break;
                    }
                }
                r0 = nextr;
                seq++;
            }
            tg += HL_VOTE_TG;
        } while (ok && tg < ntiles);
        if (!have)
            break;
    }
    if (!ok) {
        /* gave up: wait (bounded) for the copies still in flight before
         * the CTA may exit */
        for (unsigned b = seq - min(seq, (unsigned)HL_VOTE_SLOTS); b < seq; b++)
            mbar_wait_sleep(&sm.full[b % HL_VOTE_SLOTS], (b / HL_VOTE_SLOTS) & 1u);
    }
}

/* NOTE: note the bins above the threshold as peak candidates (a.cand);
 * without, the code is the plain vote and store */
template <bool UNIT, bool NOTE>
__global__ void __launch_bounds__(1024, 1)
hl_vote_kernel(hl_vote_args a)
{
    extern __shared__ __align__(128) unsigned char vote_raw[];
    VoteSmem &sm = *reinterpret_cast<VoteSmem *>(vote_raw);
    int *s_acc = reinterpret_cast<int *>(vote_raw + VOTE_FIXED);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nthr = blockDim.x, nwarps = nthr >> 5;
    const int ncons = nwarps - 1;               /* consumer warps 1..nwarps-1 */
    /* points per batch: HL_VOTE_PPW per consumer warp (at most SLOT_CAP) */
    const int batch = HL_VOTE_PPW * ncons;
    const int nslices = a.Tp / HL_SLICE;

    /* the block and its dump row start at zero (before the wait for the
     * previous launch: shared memory only); after each item the consumers
     * clear what it used */
    {
        int4 *z = reinterpret_cast<int4 *>(s_acc);
        for (int i = tid; i < (a.win_rows + 1) * (HL_SLICE / 4); i += nthr)
            z[i] = make_int4(0, 0, 0, 0);
    }
    hl_pdl_begin();
    if (tid == 0) {
        for (int i = 0; i < HL_VOTE_SLOTS; i++) {
            mbar_init(&sm.full[i], 1);
            mbar_init(&sm.empty[i], (unsigned)ncons);
        }
        for (int i = 0; i < 2; i++) {
            mbar_init(&sm.seg_full[i], 1);
            mbar_init(&sm.seg_empty[i], (unsigned)ncons);
        }
        mbar_init(&sm.cbar, (unsigned)(32 * ncons));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sm.abort = 0;
    }
    /* the only block-wide barrier: from here on the producer and the
     * consumers meet on mbarriers, every wait bounded */
    __syncthreads();
    if (warp == 0) {
        vote_producer<NOTE>(a, sm, batch);
        return;
    }

    const int cw = warp - 1;
    const int ctid = tid - 32, nct = nthr - 32;
    const unsigned acc_base = smem_u32(s_acc);
    const f2x ir = f2_pack(a.irho, a.irho);
    const int pl = lane & 7;
    int4 *src4 = reinterpret_cast<int4 *>(s_acc);
    unsigned seq = 0, nseg = 0, cpar = 0;
    /* the current item */
    DiagTab tab;
    diag_table(tab, a.cosv, a.sinv, acc_base, lane);
    int cv = CV_EXACT, vbase = 0, rows = 0, w0 = 0, k0 = 0;
    unsigned lrows = 0;
    int32_t *acc_g = nullptr;
    int nparts = 1, pslot = 0;
    int img = 0;   /* the item's image (noting candidates only) */
    while (true) {
        const int ds = (int)(nseg & 1u);
        if (!mbar_wait_ab(&sm.seg_full[ds], (nseg >> 1) & 1u, &sm.abort, a.status))
            return;
        nseg++;
        const VoteSeg &g = sm.seg[ds];
        const int item = g.item;
        const int total = g.total, b_lo = g.b_lo, b_hi = g.b_hi;
        const bool last = g.last;
        if (item >= 0 && g.first) {
            const int slice = item % nslices, win = item / nslices;
            k0 = slice * HL_SLICE;
            diag_table(tab, g.c, g.s, acc_base, lane);
            w0 = win * a.win_rows;
            rows = min(a.win_rows, g.R - w0);
            const int row_base = g.rho_min + w0;   /* rho bin of local row 0 */
            /* every column's dump row is row `rows`; the padding columns
             * (thetas >= T, cos = sin = 0) vote there or into their own
             * column, which the store writes as zero */
            lrows = (unsigned)rows;
            cv = row_base >= 1 ? CV_FLOOR
                               : (row_base + rows - 1 <= -1 ? CV_CEIL : CV_EXACT);
            vbase = cv == CV_EXACT ? row_base : RHO_MAGIC_BITS + row_base;
            acc_g = g.acc;
            nparts = g.nparts;
            pslot = g.slot;
            if (NOTE)
                img = g.img;
        }
        __syncwarp();
        if (lane == 0)
            mbar_arrive(&sm.seg_empty[ds]);
        if (item < 0)
            return;

        /* vote every point of the segment's batches, freeing each slot */
        for (int b = b_lo; b < b_hi; b++) {
            const int slot = (int)(seq % HL_VOTE_SLOTS);
            if (!mbar_wait_ab(&sm.full[slot], (seq / HL_VOTE_SLOTS) & 1u, &sm.abort,
                              a.status))
                return;
            seq++;
            /* this warp's share: points [PPW cw, PPW cw + PPW) */
            const int m = min(HL_VOTE_PPW, total - b * batch - HL_VOTE_PPW * cw);
            const float2 *pts = sm.raw[slot] + HL_VOTE_PPW * cw;
            if (cv == CV_FLOOR)
                vote_share<UNIT, CV_FLOOR>(pts, m, tab, ir, vbase, lrows, pl);
            else if (cv == CV_CEIL)
                vote_share<UNIT, CV_CEIL>(pts, m, tab, ir, vbase, lrows, pl);
            else
                vote_share<UNIT, CV_EXACT>(pts, m, tab, ir, vbase, lrows, pl);
            __syncwarp();
            if (lane == 0)
                mbar_arrive(&sm.empty[slot]);
        }
        if (!last)
            continue;

        /* the item is voted: store the block, row i of the window ->
         * acc[(w0 + i) * Tp + k0 ..], then clear it for the next item */
        if (!cons_sync(sm, cpar, a.status))
            return;
        /* a whole block goes to acc (the padding columns, thetas >= T,
         * hold dumped votes and are stored as zero; bins above the
         * image's threshold are noted as peak candidates), a part of a
         * split block to its scratch slot as it is; each thread stores and
         * clears the same elements */
        const int tp4 = a.Tp >> 2;
        const int n4 = rows * (HL_SLICE / 4);
        int4 *dst4 = nparts == 1 ? reinterpret_cast<int4 *>(acc_g) + (size_t)w0 * tp4 + (k0 >> 2)
                                 : a.scratch + (size_t)pslot * hl_slot4(a.win_rows, a.part16);
        const bool pack = nparts > 1 && a.part16;
        /* the image's peak threshold, read once (noting candidates only) */
        const int thr = NOTE ? (a.imgs ? a.imgs[img].threshold : a.img0.threshold) : 0;
        for (int i = ctid; i < n4 + HL_SLICE / 4; i += nct) {
            if (i < n4) {
                const int rr = i >> 3, q = i & 7;
                int4 v = src4[i];
                if (nparts == 1) {
                    if (k0 + 4 * q + 3 >= a.T) {
                        const int kq = k0 + 4 * q;
                        if (kq >= a.T) v.x = 0;
                        if (kq + 1 >= a.T) v.y = 0;
                        if (kq + 2 >= a.T) v.z = 0;
                        if (kq + 3 >= a.T) v.w = 0;
                    }
                    dst4[(size_t)rr * tp4 + q] = v;
                    if (NOTE) {
                        const unsigned bits = above4(v, thr, k0 + 4 * q, a.T);
                        if (bits)
                            note_cands(a.cand, img,
                                       (unsigned)(w0 + rr) * (unsigned)a.T +
                                           (unsigned)(k0 + 4 * q),
                                       bits);
                    }
                } else if (pack) {
                    reinterpret_cast<int2 *>(dst4)[i] =
                        make_int2((v.x & 0xffff) | (v.y << 16), (v.z & 0xffff) | (v.w << 16));
                } else {
                    dst4[i] = v;
                }
            }
            src4[i] = make_int4(0, 0, 0, 0);
        }
        if (!cons_sync(sm, cpar, a.status))
            return;
    }
}

/* The blocks voted in parts: block region = sum of its parts' scratch
 * slots, the padding columns (thetas >= T) stored as zero, the bins above
 * the image's threshold noted as peak candidates.  A
 * thread takes 16 bytes of every part of its region (grid.y = region): two
 * output int4 when the parts hold 16-bit counts, one otherwise; every slot
 * is read once, from L2 where the vote launch just wrote it; the parts'
 * loads go four at a time, all in flight. */
template <bool NOTE>
__global__ void __launch_bounds__(256)
hl_merge_kernel(hl_merge_args a)
{
    hl_pdl_begin();
    const hl_merge_region r = a.regs[blockIdx.y];
    const int n4 = r.rows * (HL_SLICE / 4);   /* output int4 of the region */
    int4 v0 = make_int4(0, 0, 0, 0), v1 = make_int4(0, 0, 0, 0);
    int o;   /* first output int4 of this thread */
    if (a.part16) {
        /* one 16-byte load per part: eight 16-bit counts, output int4 o and
         * o + 1 (a row holds 8, so both lie in one row); the parts' loads
         * four at a time, all four in flight (the last group predicated) */
        const int j = blockIdx.x * 256 + threadIdx.x;
        o = 2 * j;
        if (o >= n4)
            return;
        const int4 *src = a.scratch + (size_t)r.slot0 * a.slot4 + j;
        for (int p = 0; p < r.nparts; p += 4) {
            int4 q[4];
#pragma unroll
            for (int u = 0; u < 4; u++)
                q[u] = p + u < r.nparts ? __ldcg(src + (size_t)(p + u) * a.slot4)
                                        : make_int4(0, 0, 0, 0);
#pragma unroll
            for (int u = 0; u < 4; u++) {
                v0.x += q[u].x & 0xffff;
                v0.y += (unsigned)q[u].x >> 16;
                v0.z += q[u].y & 0xffff;
                v0.w += (unsigned)q[u].y >> 16;
                v1.x += q[u].z & 0xffff;
                v1.y += (unsigned)q[u].z >> 16;
                v1.z += q[u].w & 0xffff;
                v1.w += (unsigned)q[u].w >> 16;
            }
        }
    } else {
        o = blockIdx.x * 256 + threadIdx.x;
        if (o >= n4)
            return;
        const int4 *src = a.scratch + (size_t)r.slot0 * a.slot4 + o;
        for (int p = 0; p < r.nparts; p += 4) {
            int4 q[4];
#pragma unroll
            for (int u = 0; u < 4; u++)
                q[u] = p + u < r.nparts ? __ldcg(src + (size_t)(p + u) * a.slot4)
                                        : make_int4(0, 0, 0, 0);
#pragma unroll
            for (int u = 0; u < 4; u++) {
                v0.x += q[u].x;
                v0.y += q[u].y;
                v0.z += q[u].z;
                v0.w += q[u].w;
            }
        }
    }
    const int nout = a.part16 ? 2 : 1;
    for (int e = 0; e < nout; e++) {
        int4 v = e ? v1 : v0;
        const int oi = o + e;
        const int rr = oi >> 3, q = oi & 7;
        if (r.k0 + 4 * q + 3 >= a.T) {
            const int kq = r.k0 + 4 * q;
            if (kq >= a.T) v.x = 0;
            if (kq + 1 >= a.T) v.y = 0;
            if (kq + 2 >= a.T) v.z = 0;
            if (kq + 3 >= a.T) v.w = 0;
        }
        a.acc[r.off4 + (size_t)rr * a.pitch4 + q] = v;
        if (NOTE) {
            const unsigned bits =
                above4(v, a.pimgs ? a.pimgs[r.img].threshold : a.thr0, r.k0 + 4 * q, a.T);
            if (bits)
                note_cands(a.cand, r.img,
                           (unsigned)(r.w0 + rr) * (unsigned)a.T + (unsigned)(r.k0 + 4 * q), bits);
        }
    }
}

cudaError_t hl_launch_merge(const hl_merge_args *a, int max_rows, cudaStream_t s)
{
    if (a->nreg <= 0)
        return cudaSuccess;
    const int per_thread = a->part16 ? 2 : 1;   /* output int4 per thread */
    const unsigned gx =
        (unsigned)((max_rows * (HL_SLICE / 4) / per_thread + 255) / 256);
    if (a->cand.e)
        return hl_launch_pdl(hl_merge_kernel<true>, dim3(gx, (unsigned)a->nreg), dim3(256), 0, s,
                             false, *a);
    return hl_launch_pdl(hl_merge_kernel<false>, dim3(gx, (unsigned)a->nreg), dim3(256), 0, s,
                         false, *a);
}

cudaError_t hl_launch_tile_masks(const hl_vote_args *a, int nimg, size_t max_words,
                                 cudaStream_t s)
{
    if (nimg <= 0 || max_words == 0)
        return cudaSuccess;
    size_t blocks = (max_words * 32 + 255) / 256;
    if (blocks > 4096)
        blocks = 4096;
    hl_tile_mask_kernel<<<dim3((unsigned)blocks, (unsigned)nimg), 256, 0, s>>>(*a);
    return cudaGetLastError();
}

template <bool UNIT, bool NOTE>
static cudaError_t launch_vote_t(const hl_vote_args *a, int threads, int grid, size_t smem,
                                 cudaStream_t s)
{
    const cudaError_t e = cudaFuncSetAttribute(hl_vote_kernel<UNIT, NOTE>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
    if (e != cudaSuccess)
        return e;
    return hl_launch_pdl(hl_vote_kernel<UNIT, NOTE>, dim3(grid), dim3(threads), smem, s, false,
                         *a);
}

cudaError_t hl_launch_vote(const hl_vote_args *a, int threads, int grid,
                           cudaStream_t s)
{
    const size_t smem = hl_vote_smem_bytes(a->win_rows);
    const bool note = a->cand.e != nullptr;
    if (a->irho == 1.0f)
        return note ? launch_vote_t<true, true>(a, threads, grid, smem, s)
                    : launch_vote_t<true, false>(a, threads, grid, smem, s);
    return note ? launch_vote_t<false, true>(a, threads, grid, smem, s)
                : launch_vote_t<false, false>(a, threads, grid, smem, s);
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
