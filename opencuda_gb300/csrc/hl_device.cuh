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

#endif
