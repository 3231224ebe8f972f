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
 * per lane) x win_rows rho bins.  A warp takes two points per step; its 32
 * lanes add to 32 different thetas of the same point -- 32 different banks --
 * so every shared atomic instruction is conflict-free and no two lanes ever
 * hit one address (the aggregation a warp-aggregated atomic would buy is built
 * into the layout).
 *
 * Persistent CTAs take items heaviest-first from a global counter.  For an
 * item, a coarse filter marks the 128x32 compaction tiles whose rho interval
 * over the slice meets the window; runs of marked tiles are contiguous in the
 * tile-major point list, and thread 0 streams them into shared memory with
 * cp.async.bulk (TMA bulk copies of 16-byte aligned supersets of each run)
 * completing on an mbarrier, two batches in flight.  All threads then unpack
 * each batch, drop points whose own rho interval over the slice misses the
 * window, and vote.  At the end of the item the block is stored with
 * coalesced 128-byte rows into acc[R][Tp]; every bin is written exactly once,
 * so the global accumulator needs no clearing.
 *
 * Bounds: a point votes without per-vote checks only when its rho interval
 * over the slice lies, with three bins of slack, inside the window; a point
 * that straddles the window checks every vote (predicated red.shared), lanes
 * beyond T add into a private sink word, and mbarrier waits are bounded (a
 * time-out sets a status bit that the host reads with the result; the CTA
 * keeps the same barrier sequence and stops taking items).
 *
 * Instruction budget per point and warp on the interior path: one shared
 * load per two points, two multiplies, one add, one float->int truncation,
 * one address multiply-add and one red.shared -- the truncation (16 per
 * SM-clock) is the binding pipe, about half the measured red.shared rate.
 */
#include "hl_internal.h"

#define FULL 0xffffffffu
#define RAWCAP (HL_VOTE_CHUNK + 6 * HL_VOTE_PIECES + 32)
#define MBAR_SPIN_LIMIT (1 << 22)

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

/* rho values of the two points (x0, y0), (x1, y1) of a pair record
 * {x0, x1, y0, y1} for this lane's (c, s) */
template <bool UNIT>
__device__ __forceinline__ void rho_pair(const float4 &q, float c, float s,
                                         float irho, int &r0, int &r1)
{
    r0 = rho_of<UNIT>(q.x, q.z, c, s, irho);
    r1 = rho_of<UNIT>(q.y, q.w, c, s, irho);
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
/* bounded wait for the phase with the given parity; false on time-out */
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar,
                                          unsigned parity)
{
    const unsigned a = smem_u32(bar);
    for (int i = 0; i < MBAR_SPIN_LIMIT; i++) {
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

/* Conservative test: can any point of tile t vote into rho bins
 * [lo_bin, hi_bin] for a theta in [th0, th1]?  rho(x, y, th) is linear in
 * (x, y) for fixed th, so its extremes over the tile lie at the corners; over
 * th in [th0, th1] (within [0, pi)) a corner's value |p| cos(th - phi), phi in
 * [0, pi/2], has no interior minimum and an interior maximum |p| <= x + y only
 * when phi lies between th0 and th1.  Three bins of slack cover rounding. */
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
            hi = fmaxf(hi, x + y);
        mx = fmaxf(mx, hi);
    }
    mn = mn * irho - 3.0f;
    mx = mx * irho + 3.0f;
    return mn <= hi_bin && mx >= lo_bin;
}

struct VoteSmem {
    unsigned long long mbar[2];
    int item;
    int nruns;
    int nin[3];                       /* interior points kept, per batch */
    int nst[3];                       /* straddling points kept, per batch */
    int np[2];
    int total[2];
    int timeout;
    int pc_src[2][HL_VOTE_PIECES];    /* first point copied (multiple of 4) */
    int pc_roff[2][HL_VOTE_PIECES];   /* offset in raw[slot] */
    int pc_skip[2][HL_VOTE_PIECES];   /* leading points copied but not used */
    int pc_base[2][HL_VOTE_PIECES + 1];
    unsigned mask[HL_VOTE_TG / 32];
    int run_s[HL_VOTE_TG / 2 + 1];
    int run_e[HL_VOTE_TG / 2 + 1];
    int sink[HL_SLICE];               /* votes of lanes past the last theta */
    alignas(16) unsigned raw[2][RAWCAP];
    /* unpacked points as pair records {x0, x1, y0, y1} */
    alignas(16) float4 cin[2][HL_VOTE_CHUNK / 2 + 1];
    alignas(16) float4 cst[2][HL_VOTE_CHUNK / 2 + 1];
};

#define VOTE_FIXED ((sizeof(VoteSmem) + 127) / 128 * 128)

size_t hl_vote_smem_bytes(int win_rows)
{
    return VOTE_FIXED + (size_t)win_rows * HL_SLICE * sizeof(int);
}

/* one vote: shared-memory reduction without a returned value */
__device__ __forceinline__ void red_smem(unsigned addr)
{
    asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(addr));
}
/* one vote if the window-relative row rl is below lim */
__device__ __forceinline__ void red_smem_if(unsigned addr, unsigned rl,
                                            unsigned lim)
{
    asm volatile("{ .reg .pred p; setp.lt.u32 p, %1, %2; "
                 "@p red.shared.add.u32 [%0], 1; }" ::"r"(addr),
                 "r"(rl), "r"(lim));
}

/* Producer (thread 0): form the next batch of up to HL_VOTE_CHUNK points from
 * the run list and start its bulk copies into raw[slot].  State: run index r
 * and point cursor pos.  Source and destination of every copy are 16-byte
 * aligned (whole groups of 4 points) and the point list is allocated with at
 * least 4 entries of slack, so the rounded-up tail stays in bounds. */
__device__ void produce(VoteSmem &sm, int slot, const uint32_t *pts, int &r,
                        int &pos)
{
    int total = 0, np = 0, roff = 0;
    const int nruns = sm.nruns;
    while (np < HL_VOTE_PIECES && total < HL_VOTE_CHUNK && r < nruns) {
        if (pos >= sm.run_e[r]) {
            r++;
            if (r < nruns)
                pos = sm.run_s[r];
            continue;
        }
        const int take = min(sm.run_e[r] - pos, HL_VOTE_CHUNK - total);
        const int a0 = pos & ~3;
        const int a1 = (pos + take + 3) & ~3;
        sm.pc_src[slot][np] = a0;
        sm.pc_roff[slot][np] = roff;
        sm.pc_skip[slot][np] = pos - a0;
        sm.pc_base[slot][np] = total;
        roff += a1 - a0;
        total += take;
        pos += take;
        np++;
    }
    sm.pc_base[slot][np] = total;
    sm.np[slot] = np;
    sm.total[slot] = total;
    if (total > 0) {
        mbar_expect_tx(&sm.mbar[slot], (unsigned)roff * 4u);
        for (int p = 0; p < np; p++) {
            const int end = (p + 1 < np) ? sm.pc_roff[slot][p + 1] : roff;
            const int nb = end - sm.pc_roff[slot][p];
            bulk_g2s(&sm.raw[slot][sm.pc_roff[slot][p]], pts + sm.pc_src[slot][p],
                     (unsigned)nb * 4u, &sm.mbar[slot]);
        }
    }
}

/* append a point to a pair-record list with a warp-aggregated counter */
__device__ __forceinline__ void append_point(bool take, float x, float y,
                                             int *counter, float *list)
{
    const int lane = threadIdx.x & 31;
    const unsigned bm = __ballot_sync(FULL, take);
    if (!bm)
        return;
    const int leader = __ffs(bm) - 1;
    int base = 0;
    if (lane == leader)
        base = atomicAdd(counter, __popc(bm));
    base = __shfl_sync(FULL, base, leader);
    if (take) {
        const int q = base + __popc(bm & ((1u << lane) - 1u));
        list[(q >> 1) * 4 + (q & 1)] = x;
        list[(q >> 1) * 4 + 2 + (q & 1)] = y;
    }
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
    const int nslices = a.Tp / HL_SLICE;

    if (tid == 0) {
        mbar_init(&sm.mbar[0], 1);
        mbar_init(&sm.mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sm.timeout = 0;
    }
    unsigned use0 = 0u, use1 = 0u;   /* completed phases of mbar[0], mbar[1] */
    __syncthreads();

    while (true) {
        if (tid == 0) {
            const unsigned t = atomicAdd(a.work, 1u) - a.work_base;
            sm.item = (t < (unsigned)a.nitems) ? a.item_order[t] : -1;
        }
        __syncthreads();
        const int item = sm.item;
        if (item < 0 || sm.timeout)
            break;
        const int slice = item % nslices, win = item / nslices;
        const int k0 = slice * HL_SLICE, k = k0 + lane;
        const float c = a.cosv[k], s = a.sinv[k];   /* table padded to Tp */
        const int w0 = win * a.win_rows;
        const int rows = min(a.win_rows, a.R - w0);
        const int row_base = a.rho_min + w0;       /* rho bin of local row 0 */
        const bool kv = k < a.T;
        const unsigned lrows = kv ? (unsigned)rows : 0u;
        const int klast = min(k0 + HL_SLICE - 1, a.T - 1);
        const float c0 = a.cosv[k0], s0 = a.sinv[k0];
        const float c1 = a.cosv[klast], s1 = a.sinv[klast];
        const float lo_bin = (float)row_base;
        const float hi_bin = (float)(row_base + rows - 1);
        const bool filter = a.nwin > 1;
        /* shared addresses: bin row rl of this lane is acc_l + rl * 128;
         * interior votes index by rho directly (base folded), and lanes past
         * the last theta vote into their own sink word */
        const unsigned acc_l = smem_u32(s_acc) + 4u * lane;
        const unsigned in_mul = kv ? 128u : 0u;
        const unsigned in_base = kv ? acc_l - 128u * (unsigned)row_base
                                    : smem_u32(&sm.sink[lane]);

        {
            int4 *z = reinterpret_cast<int4 *>(s_acc);
            const int4 zero = make_int4(0, 0, 0, 0);
            for (int i = tid; i < rows * (HL_SLICE / 4); i += nthr)
                z[i] = zero;
        }

        for (int tg = 0; tg < a.ntiles; tg += HL_VOTE_TG) {
            const int tg_n = min(HL_VOTE_TG, a.ntiles - tg);
            /* coarse filter: one bit per tile of the group */
            for (int wd = warp; wd < HL_VOTE_TG / 32; wd += nwarps) {
                const int tl = wd * 32 + lane;
                bool hit = false;
                if (tl < tg_n)
                    hit = !filter || tile_hits(tg + tl, a.tiles_x, a.w, a.h, c0,
                                               s0, c1, s1, lo_bin, hi_bin,
                                               a.irho);
                const unsigned m = __ballot_sync(FULL, hit);
                if (lane == 0)
                    sm.mask[wd] = m;
            }
            __syncthreads();
            /* runs of marked tiles -> point ranges (warp 0) */
            if (warp == 0) {
                const unsigned m = sm.mask[lane];
                const unsigned prev = __shfl_up_sync(FULL, m, 1);
                const unsigned next = __shfl_down_sync(FULL, m, 1);
                const unsigned carry_in = (lane > 0) ? (prev >> 31) : 0u;
                const unsigned carry_out = (lane < 31) ? (next & 1u) : 0u;
                unsigned starts = m & ~((m << 1) | carry_in);
                unsigned ends = m & ~((m >> 1) | (carry_out << 31));
                const int ns = __popc(starts), ne = __popc(ends);
                int bs = ns, be = ne;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t1 = __shfl_up_sync(FULL, bs, o);
                    const int t2 = __shfl_up_sync(FULL, be, o);
                    if (lane >= o) {
                        bs += t1;
                        be += t2;
                    }
                }
                bs -= ns;
                be -= ne;
                while (starts) {
                    const int b = __ffs(starts) - 1;
                    starts &= starts - 1;
                    sm.run_s[bs++] = a.tile_off[tg + lane * 32 + b];
                }
                while (ends) {
                    const int b = __ffs(ends) - 1;
                    ends &= ends - 1;
                    sm.run_e[be++] = a.tile_off[tg + lane * 32 + b + 1];
                }
                if (lane == 31)
                    sm.nruns = bs;
            }
            __syncthreads();

            /* stream the runs through shared memory, two batches in flight */
            int r = 0, pos = (sm.nruns > 0) ? sm.run_s[0] : 0;
            if (tid == 0) {
                sm.nin[0] = sm.nin[1] = sm.nin[2] = 0;
                sm.nst[0] = sm.nst[1] = sm.nst[2] = 0;
                produce(sm, 0, a.pts, r, pos);
                produce(sm, 1, a.pts, r, pos);
            }
            __syncthreads();
            for (int b = 0;; b++) {
                const int slot = b & 1;
                const int total = sm.total[slot];
                if (total == 0)
                    break;
                const unsigned par = (slot ? use1 : use0) & 1u;
                const bool ok = mbar_wait(&sm.mbar[slot], par);
                if (slot)
                    use1++;
                else
                    use0++;
                if (!ok && lane == 0) {
                    /* the batch never arrived: flag it and carry on with the
                     * same barriers (votes stay inside the window, so the
                     * result is only wrong, and the call reports it) */
                    sm.timeout = 1;
                    atomicOr(a.status, HL_ST_VOTE_TIMEOUT);
                }
                /* unpack; each point's own rho interval over the slice sorts
                 * it into interior (every vote inside the window), straddling
                 * (some inside) or dropped */
                const int np = sm.np[slot];
                const int cnt_i = b % 3;
                float *lin = reinterpret_cast<float *>(sm.cin[slot]);
                float *lst = reinterpret_cast<float *>(sm.cst[slot]);
                for (int j0 = 0; j0 < total; j0 += nthr) {
                    const int j = j0 + tid;
                    bool inner = false, strad = false;
                    float x = 0.f, y = 0.f;
                    if (j < total) {
                        int p = 0;
                        while (p + 1 < np && sm.pc_base[slot][p + 1] <= j)
                            p++;
                        const unsigned u =
                            sm.raw[slot][sm.pc_roff[slot][p] + sm.pc_skip[slot][p] +
                                         (j - sm.pc_base[slot][p])];
                        x = (float)(u & 0xffffu);
                        y = (float)(u >> 16);
                        const float f0 = x * c0 + y * s0;
                        const float f1 = x * c1 + y * s1;
                        float lo = fminf(f0, f1), hi = fmaxf(f0, f1);
                        const float tol = 1e-3f * (x + y) + 1e-3f;
                        if (c0 * y - s0 * x >= -tol && x * s1 - y * c1 >= -tol)
                            hi = fmaxf(hi, x + y);
                        lo = lo * a.irho;
                        hi = hi * a.irho;
                        inner = (lo - 3.0f >= lo_bin) && (hi + 3.0f <= hi_bin);
                        strad = !inner && (lo - 3.0f <= hi_bin) && (hi + 3.0f >= lo_bin);
                    }
                    append_point(inner, x, y, &sm.nin[cnt_i], lin);
                    append_point(strad, x, y, &sm.nst[cnt_i], lst);
                }
                __syncthreads();
                const int n_in = sm.nin[cnt_i], n_st = sm.nst[cnt_i];
                if (tid == 0) {
                    /* counters of batch b + 2: last read (for batch b - 1)
                     * before this step's barrier by every thread */
                    sm.nin[(b + 2) % 3] = 0;
                    sm.nst[(b + 2) % 3] = 0;
                    produce(sm, slot, a.pts, r, pos);
                }
                /* interior points: every vote lands in the window */
                {
                    const int npairs = n_in >> 1;
                    const float4 *c4 = sm.cin[slot];
                    int p = warp;
                    for (; p + nwarps < npairs; p += 2 * nwarps) {
                        const float4 qa = c4[p];
                        const float4 qb = c4[p + nwarps];
                        int r0, r1, r2, r3;
                        rho_pair<UNIT>(qa, c, s, a.irho, r0, r1);
                        rho_pair<UNIT>(qb, c, s, a.irho, r2, r3);
                        red_smem((unsigned)r0 * in_mul + in_base);
                        red_smem((unsigned)r1 * in_mul + in_base);
                        red_smem((unsigned)r2 * in_mul + in_base);
                        red_smem((unsigned)r3 * in_mul + in_base);
                    }
                    if (p < npairs) {
                        int r0, r1;
                        rho_pair<UNIT>(c4[p], c, s, a.irho, r0, r1);
                        red_smem((unsigned)r0 * in_mul + in_base);
                        red_smem((unsigned)r1 * in_mul + in_base);
                    }
                    if ((n_in & 1) && warp == nwarps - 1) {
                        const float4 q = c4[npairs];
                        const int r0 = rho_of<UNIT>(q.x, q.z, c, s, a.irho);
                        red_smem((unsigned)r0 * in_mul + in_base);
                    }
                }
                /* straddling points: only the lanes inside the window vote */
                {
                    const int npairs = n_st >> 1;
                    const float4 *c4 = sm.cst[slot];
                    int p = nwarps - 1 - warp;   /* other end of the warp range */
                    for (; p < npairs; p += nwarps) {
                        int r0, r1;
                        rho_pair<UNIT>(c4[p], c, s, a.irho, r0, r1);
                        const unsigned l0 = (unsigned)(r0 - row_base);
                        const unsigned l1 = (unsigned)(r1 - row_base);
                        red_smem_if(acc_l + 128u * l0, l0, lrows);
                        red_smem_if(acc_l + 128u * l1, l1, lrows);
                    }
                    if ((n_st & 1) && warp == 0) {
                        const float4 q = c4[npairs];
                        const int r0 = rho_of<UNIT>(q.x, q.z, c, s, a.irho);
                        const unsigned l0 = (unsigned)(r0 - row_base);
                        red_smem_if(acc_l + 128u * l0, l0, lrows);
                    }
                }
            }
            __syncthreads();
        }

        /* store the block: row i of the window -> acc[(w0 + i) * Tp + k0 ..] */
        int4 *dst4 = reinterpret_cast<int4 *>(a.acc);
        const int4 *src4 = reinterpret_cast<const int4 *>(s_acc);
        const int tp4 = a.Tp >> 2;
        for (int i = tid; i < rows * (HL_SLICE / 4); i += nthr) {
            const int rr = i >> 3, q = i & 7;
            dst4[(size_t)(w0 + rr) * tp4 + (k0 >> 2) + q] = src4[i];
        }
        __syncthreads();
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
