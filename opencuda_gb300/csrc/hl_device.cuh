/*
 * hl_device.cuh -- device helpers shared by the vote kernels (full
 * accumulator and proposal windows).
 */
#ifndef HL_DEVICE_CUH
#define HL_DEVICE_CUH

#include "hl_internal.h"

/* The vote rule (okano_3_0/HoughLine.cu:115-121): rho = trunc(fl(fl(x cos) +
 * fl(y sin))), each product times irho when derho != 1; no contraction. */
template <bool UNIT>
__device__ __forceinline__ float rho_f(float x, float y, float c, float s,
                                       float irho)
{
    float a = __fmul_rn(x, c);
    float b = __fmul_rn(y, s);
    if (!UNIT) {
        a = __fmul_rn(a, irho);
        b = __fmul_rn(b, irho);
    }
    return __fadd_rn(a, b);
}
template <bool UNIT>
__device__ __forceinline__ int rho_of(float x, float y, float c, float s,
                                      float irho)
{
    return __float2int_rz(rho_f<UNIT>(x, y, c, s, irho));
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
/* CV_SIGN: truncation for a window that holds rows of both signs without the
 * conversion pipe: floor (round toward zero of v + M) where v >= 0, ceil
 * (round up) where v < 0, picked by the sign bit of v with one bitwise
 * select; the base is then bits(M) plus the rho of row 0, as for CV_FLOOR. */
enum { CV_EXACT = 0, CV_FLOOR = 1, CV_CEIL = 2, CV_SIGN = 3 };

/* one vote, no returned value */
__device__ __forceinline__ void red_smem(unsigned addr)
{
    asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(addr));
}

/* ---- packed f32x2 arithmetic ------------------------------------------ *
 * Two lanes of a 64-bit register pair per instruction.  The products are
 * formed as fma.rn(a, b, +0): exactly fl(a*b) for the finite operands here
 * (a -0 product becomes +0, which no later sum or truncation can tell
 * apart).  A plain mul.rn.f32x2 followed by add.rn.f32x2 is contracted by
 * ptxas into one fused multiply-add, which changes rho in a small fraction
 * of votes; the fma form is never contracted (checked on the GPU against
 * the scalar __fmul_rn/__fadd_rn rule for every (x, y) of a 4096 x 4096
 * image at T = 720: no difference). */
typedef unsigned long long f2x;
__device__ __forceinline__ f2x f2_pack(float a, float b)
{
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2x r, unsigned &a, unsigned &b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=r"(a), "=r"(b) : "l"(r));
}
__device__ __forceinline__ f2x f2_mul(f2x a, f2x b)
{
    f2x d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(0ull));
    return d;
}
__device__ __forceinline__ f2x f2_add(f2x a, f2x b)
{
    f2x d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_add_rz(f2x a, f2x b)
{
    f2x d;
    asm("add.rz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_add_rp(f2x a, f2x b)
{
    f2x d;
    asm("add.rp.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

/* Diagonal vote schedule.  A consumer warp votes 8 points at a time, each
 * point on 4 lanes: lane = p + 8 j (point p, theta group j).  At step i the
 * lane votes theta column 8 j + (p + i) % 8 of the slice, so at every step
 * the 32 lanes address 32 different columns -- 32 different banks, whatever
 * rows their points reach -- and over the 8 steps every point votes all 32
 * thetas.  A lane loads its point once per 8 votes (one shared-memory
 * wavefront for the warp's 8 points), where a broadcast load per point
 * would cost as many wavefronts as the atomics themselves: the shared
 * pipe serves loads, shuffles and reductions alike at about one wavefront
 * per SM-clock.  Each lane keeps its 8 columns' cos/sin as f32x2 pairs of
 * consecutive steps and the columns' shared-memory addresses. */
struct DiagTab {
    f2x c[4], s[4];        /* cos / sin of the lane's columns, steps (2i, 2i + 1) */
    unsigned col[8];       /* address of the lane's column at step i, row 0 */
};

__device__ __forceinline__ void diag_table(DiagTab &t, const float *cs, const float *sn,
                                           unsigned acc_base, int lane)
{
    const int p = lane & 7, j = lane >> 3;
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
        const int c0 = 8 * j + ((p + i) & 7), c1 = 8 * j + ((p + i + 1) & 7);
        t.c[i / 2] = f2_pack(cs[c0], cs[c1]);
        t.s[i / 2] = f2_pack(sn[c0], sn[c1]);
        t.col[i] = acc_base + 4u * (unsigned)c0;
        t.col[i + 1] = acc_base + 4u * (unsigned)c1;
    }
}

/* The 8 steps of one point (x, y) on this lane.  rho per the vote rule
 * (okano_3_0/HoughLine.cu:115-121), the row relative to the window clamped
 * to the dump row `lim`; float -> integer by the magic constant (CV_FLOOR /
 * CV_CEIL, CV_SIGN, see RHO_MAGIC) or by the exact conversion (CV_EXACT). */
template <bool UNIT, int CV>
__device__ __forceinline__ void diag_point(float x, float y, const DiagTab &t, f2x ir,
                                           int base, unsigned lim)
{
    const f2x X = f2_pack(x, x), Y = f2_pack(y, y);
    const f2x M = f2_pack(RHO_MAGIC, RHO_MAGIC);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        f2x a = f2_mul(X, t.c[i]), b = f2_mul(Y, t.s[i]);
        if (!UNIT) {
            a = f2_mul(a, ir);
            b = f2_mul(b, ir);
        }
        const f2x v = f2_add(a, b);
        unsigned r0, r1;
        if (CV == CV_FLOOR) {
            f2_unpack(f2_add_rz(v, M), r0, r1);
        } else if (CV == CV_CEIL) {
            f2_unpack(f2_add_rp(v, M), r0, r1);
        } else if (CV == CV_SIGN) {
            unsigned u0, u1, f0, f1, c0, c1;
            f2_unpack(v, u0, u1);
            f2_unpack(f2_add_rz(v, M), f0, f1);
            f2_unpack(f2_add_rp(v, M), c0, c1);
            const unsigned s0 = (unsigned)((int)u0 >> 31), s1 = (unsigned)((int)u1 >> 31);
            r0 = (c0 & s0) | (f0 & ~s0);
            r1 = (c1 & s1) | (f1 & ~s1);
        } else {
            unsigned u0, u1;
            f2_unpack(v, u0, u1);
            r0 = (unsigned)__float2int_rz(__uint_as_float(u0));
            r1 = (unsigned)__float2int_rz(__uint_as_float(u1));
        }
        red_smem(t.col[2 * i] + 128u * min(r0 - (unsigned)base, lim));
        red_smem(t.col[2 * i + 1] + 128u * min(r1 - (unsigned)base, lim));
    }
}


/* Notes the bins of one int4 of counts whose bit is set in bits (bin
 * idx0 + j for bit j, j < 4) as peak candidates of image img; once the list
 * is full (the peak pass then scans every accumulator) a bin costs one
 * load. */
__device__ __forceinline__ void note_cands(const hl_cand_list &c, int img, unsigned idx0,
                                           unsigned bits)
{
    if (*(volatile int *)c.count >= c.cap)
        return;
    while (bits) {
        const int j = __ffs(bits) - 1;
        bits &= bits - 1;
        const int pos = atomicAdd(c.count, 1);
        if (pos < c.cap)
            c.e[pos] = ((unsigned long long)(unsigned)img << 32) | (idx0 + (unsigned)j);
    }
}

/* bits of the bins of v above thr, bins kq + j >= T (padding) left out */
__device__ __forceinline__ unsigned above4(const int4 &v, int thr, int kq, int T)
{
    unsigned b = (unsigned)(v.x > thr) | ((unsigned)(v.y > thr) << 1) |
                 ((unsigned)(v.z > thr) << 2) | ((unsigned)(v.w > thr) << 3);
    if (kq + 3 >= T)
        b &= (T > kq) ? (1u << (T - kq)) - 1u : 0u;
    return b;
}

#endif
