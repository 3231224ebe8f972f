/*
 * hl_stage_f.cu -- the entry points either side of the plain path:
 *
 *   hl_draw_kernel      houghLineImg's line rendering (okano_3_0/HoughLine.cu:
 *                       216-249): output pixel (c, r) of the ROI becomes 255
 *                       when (int)(fl(c*cos a) + fl(r*sin a)) equals a line's
 *                       distance.  cos/sin of each line angle are evaluated
 *                       once per CTA with CUDA's cosf/sinf (the values the
 *                       reference evaluates per pixel) and kept in shared
 *                       memory; the kernel is output-bound (one byte store
 *                       per lit pixel, one read-modify per ROI pixel).
 *   hl_real_line_kernel realLine's segment check (:252-284): edge pixels of the
 *                       segment's bounding box (grown by delta) within delta
 *                       of the segment are counted.  Only the box is
 *                       launched, not the whole image.
 */
#include "hl_internal.h"

#include <math.h>

#define FULL 0xffffffffu
#define DRAW_MAX_LINES 1024

__global__ void hl_draw_kernel(uint8_t *out, long pitch, int w, int h,
                               const hl_line *lines, int nlines, float irho,
                               int unit)
{
    __shared__ float s_c[DRAW_MAX_LINES], s_s[DRAW_MAX_LINES];
    __shared__ int s_d[DRAW_MAX_LINES];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nthr = blockDim.x * blockDim.y;
    const int n = min(nlines, DRAW_MAX_LINES);
    for (int i = tid; i < n; i += nthr) {
        const float a = lines[i].angle;
        s_c[i] = cosf(a);
        s_s[i] = sinf(a);
        s_d[i] = lines[i].distance;
    }
    __syncthreads();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (c >= w || r >= h)
        return;
    const float fc = (float)c, fr = (float)r;
    for (int i = 0; i < n; i++) {
        float x = __fmul_rn(fc, s_c[i]);
        float y = __fmul_rn(fr, s_s[i]);
        if (!unit) {
            x = __fmul_rn(x, irho);
            y = __fmul_rn(y, irho);
        }
        if (__float2int_rz(__fadd_rn(x, y)) == s_d[i]) {
            out[(size_t)r * pitch + c] = 255;
            break;
        }
    }
}

cudaError_t hl_launch_draw(uint8_t *out, long pitch, int w, int h,
                           const hl_line *lines, int nlines, int derho,
                           cudaStream_t s)
{
    if (nlines <= 0 || w <= 0 || h <= 0)
        return cudaSuccess;
    /* okano_3_0/HoughLine.cu:230: float irho = 1.0f / derho, derho an int */
    const float irho = 1.0f / (float)derho;
    dim3 block(32, 8);
    dim3 grid((w + 31) / 32, (h + 7) / 8);
    for (int first = 0; first < nlines; first += DRAW_MAX_LINES) {
        /* lines beyond one CTA's table are drawn by further passes; a pixel
         * lit by an earlier pass stays 255 either way */
        hl_draw_kernel<<<grid, block, 0, s>>>(out, pitch, w, h, lines + first,
                                              min(nlines - first, DRAW_MAX_LINES),
                                              irho, derho == 1);
    }
    return cudaGetLastError();
}

__global__ void hl_real_line_kernel(const uint8_t *img, long pitch, int w, int h,
                                    int x1, int y1, int x2, int y2, int bx0,
                                    int by0, int bx1, int by1, int delta,
                                    double len, int *count)
{
    const int cx = bx0 + blockIdx.x * blockDim.x + threadIdx.x;
    const int ry = by0 + blockIdx.y * blockDim.y + threadIdx.y;
    int hit = 0;
    if (cx <= bx1 && ry <= by1 && cx < w && ry < h && cx >= 0 && ry >= 0) {
        if (img[(size_t)ry * pitch + cx] == 255) {
            /* okano_3_0/HoughLine.cu:275: |cross| / |segment| in double,
             * stored as float, compared with the int delta */
            int cr = abs((x2 - x1) * (ry - y1) - (cx - x1) * (y2 - y1));
            float dis = __double2float_rn(__ddiv_rn((double)cr, len));
            hit = dis < (float)delta;
        }
    }
    const unsigned b = __ballot_sync(FULL, hit);
    if ((threadIdx.x & 31) == 0 && b)
        atomicAdd(count, __popc(b));
}

cudaError_t hl_launch_real_line(const uint8_t *img, long pitch, int w, int h,
                                int x1, int y1, int x2, int y2, int delta,
                                int *count, cudaStream_t s)
{
    const int xmin = min(x1, x2), xmax = max(x1, x2);
    const int ymin = min(y1, y2), ymax = max(y1, y2);
    /* okano_3_0/HoughLine.cu:266-267: cx in [xmin - delta, xmax + delta] */
    const int bx0 = max(xmin - delta, 0), bx1 = min(xmax + delta, w - 1);
    const int by0 = max(ymin - delta, 0), by1 = min(ymax + delta, h - 1);
    if (bx1 < bx0 || by1 < by0)
        return cudaSuccess;
    const double len = sqrt((double)(x2 - x1) * (x2 - x1) * 1.0 +
                            (double)(y2 - y1) * (y2 - y1));
    dim3 block(32, 8);
    dim3 grid((bx1 - bx0 + 32) / 32, (by1 - by0 + 8) / 8);
    hl_real_line_kernel<<<grid, block, 0, s>>>(img, pitch, w, h, x1, y1, x2, y2,
                                               bx0, by0, bx1, by1, delta, len,
                                               count);
    return cudaGetLastError();
}
