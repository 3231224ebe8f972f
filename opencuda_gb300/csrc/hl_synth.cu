/*
 * hl_synth.cu -- the seeded scene generator of synth.c on the GPU, for the
 * proposal network's training data: one CTA per image; thread 0 replays the
 * scene's random stream (segment endpoints with their rejection loop, Bezier
 * control points) in the host generator's order, then the warps draw the
 * segments and curves and all threads add the salt.  Every write sets a
 * pixel to 255, so the drawing order does not matter and the bytes equal
 * hl_synth_scene's.
 */
#include "hl_internal.h"
#include "hl_synth.h"

#define SY_MAX_SEG 256
#define SY_MAX_BEZ 32

__device__ __forceinline__ uint64_t d_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t d_next64(uint64_t *s)
{
    *s += 0x9E3779B97F4A7C15ull;
    return d_mix64(*s);
}

/* uniform integer in [lo, hi], the high word of a 64 x 64 product */
__device__ __forceinline__ long long d_urange(uint64_t *s, long long lo, long long hi)
{
    if (hi <= lo)
        return lo;
    const uint64_t span = (uint64_t)(hi - lo) + 1u;
    return lo + (long long)__umul64hi(d_next64(s), span);
}

__device__ void d_bresenham(uint8_t *img, long pitch, int w, int h, int x0,
                            int y0, int x1, int y1)
{
    int dx = x1 > x0 ? x1 - x0 : x0 - x1;
    int dy = y1 > y0 ? y0 - y1 : y1 - y0;
    int sx = x0 < x1 ? 1 : -1;
    int sy = y0 < y1 ? 1 : -1;
    int err = dx + dy;
    for (;;) {
        if (x0 >= 0 && y0 >= 0 && x0 < w && y0 < h)
            img[(long)y0 * pitch + x0] = 255;
        if (x0 == x1 && y0 == y1)
            break;
        int e2 = 2 * err;
        if (e2 >= dy) {
            err += dy;
            x0 += sx;
        }
        if (e2 <= dx) {
            err += dx;
            y0 += sy;
        }
    }
}

__device__ void d_bezier(uint8_t *img, long pitch, int w, int h, const int *c)
{
    const long long px[3] = {c[0], c[2], c[4]}, py[3] = {c[1], c[3], c[5]};
    long long n = llabs(px[1] - px[0]) + llabs(py[1] - py[0]) +
                  llabs(px[2] - px[1]) + llabs(py[2] - py[1]);
    if (n < 1)
        n = 1;
    const long long n2 = n * n;
    int lx = (int)px[0], ly = (int)py[0];
    for (long long i = 1; i <= n; i++) {
        const long long a = (n - i) * (n - i), b = 2 * (n - i) * i, cc = i * i;
        const int x = (int)((a * px[0] + b * px[1] + cc * px[2] + n2 / 2) / n2);
        const int y = (int)((a * py[0] + b * py[1] + cc * py[2] + n2 / 2) / n2);
        d_bresenham(img, pitch, w, h, lx, ly, x, y);
        lx = x;
        ly = y;
    }
}

__global__ void __launch_bounds__(256)
hl_synth_kernel(const hl_scene_params *ps, const hl_image_desc *outs)
{
    __shared__ int seg[SY_MAX_SEG][4];
    __shared__ int segok[SY_MAX_SEG];
    __shared__ int bez[SY_MAX_BEZ][6];
    const hl_scene_params p = ps[blockIdx.x];
    const hl_image_desc o = outs[blockIdx.x];
    const int w = p.width, h = p.height;
    uint8_t *img = const_cast<uint8_t *>(o.data);   /* the output image */
    const long pitch = (long)o.pitch;
    const int nseg = min(p.nseg, SY_MAX_SEG), nbez = min(p.nbezier, SY_MAX_BEZ);
    for (long i = threadIdx.x; i < (long)w * h; i += blockDim.x)
        img[(i / w) * pitch + (i % w)] = 0;
    if (threadIdx.x == 0) {
        uint64_t s = p.seed * 0xD1342543DE82EF95ull + 0x1234567ull;
        long long lmin = p.len_min, lmax = p.len_max;
        if (lmax < lmin)
            lmax = lmin;
        const long long lmin2 = lmin * lmin, lmax2 = lmax * lmax;
        for (int i = 0; i < p.nseg; i++) {
            int x0 = 0, y0 = 0, x1 = 0, y1 = 0, ok = 0;
            for (int attempt = 0; attempt < 64 && !ok; attempt++) {
                x0 = (int)d_urange(&s, 0, w - 1);
                y0 = (int)d_urange(&s, 0, h - 1);
                for (int t = 0; t < 256; t++) {
                    const long long dx = d_urange(&s, -lmax, lmax);
                    const long long dy = d_urange(&s, -lmax, lmax);
                    const long long l2 = dx * dx + dy * dy;
                    if (l2 < lmin2 || l2 > lmax2)
                        continue;
                    if (x0 + dx < 0 || x0 + dx >= w || y0 + dy < 0 || y0 + dy >= h)
                        continue;
                    x1 = (int)(x0 + dx);
                    y1 = (int)(y0 + dy);
                    ok = 1;
                    break;
                }
            }
            if (i < SY_MAX_SEG) {
                seg[i][0] = x0;
                seg[i][1] = y0;
                seg[i][2] = x1;
                seg[i][3] = y1;
                segok[i] = ok;
            }
        }
        for (int i = 0; i < p.nbezier; i++) {
            int c[6];
            for (int k = 0; k < 3; k++) {
                c[2 * k] = (int)d_urange(&s, 0, w - 1);
                c[2 * k + 1] = (int)d_urange(&s, 0, h - 1);
            }
            if (i < SY_MAX_BEZ)
                for (int k = 0; k < 6; k++)
                    bez[i][k] = c[k];
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nseg; i += blockDim.x)
        if (segok[i])
            d_bresenham(img, pitch, w, h, seg[i][0], seg[i][1], seg[i][2], seg[i][3]);
    for (int i = threadIdx.x; i < nbez; i += blockDim.x)
        d_bezier(img, pitch, w, h, bez[i]);
    if (p.salt_ppm > 0) {
        const uint64_t key = d_mix64(p.seed ^ 0x5A17C0DEull);
        for (long i = threadIdx.x; i < (long)w * h; i += blockDim.x) {
            const long y = i / w, x = i % w;
            const uint64_t base = key + (uint64_t)y * (uint64_t)w * 0x9E3779B97F4A7C15ull;
            const uint64_t r = d_mix64(base + (uint64_t)x * 0x9E3779B97F4A7C15ull);
            if ((r % 1000000u) < (uint64_t)p.salt_ppm)
                img[y * pitch + x] = 255;
        }
    }
}

extern "C" int hl_synth_scenes_device(const hl_scene_params *params, int n,
                                      const hl_image_desc *outs, void *stream)
{
    if (!params || !outs)
        return HL_NULL_POINTER;
    if (n <= 0)
        return HL_INVALID_DATA;
    for (int i = 0; i < n; i++) {
        if (!outs[i].data)
            return HL_NULL_POINTER;
        if (params[i].width <= 0 || params[i].height <= 0 ||
            outs[i].width < params[i].width || outs[i].height < params[i].height ||
            outs[i].pitch < (size_t)params[i].width || params[i].nseg > SY_MAX_SEG ||
            params[i].nbezier > SY_MAX_BEZ)
            return HL_INVALID_DATA;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    hl_scene_params *dp = nullptr;
    hl_image_desc *dd = nullptr;
    if (cudaMallocAsync(&dp, sizeof(hl_scene_params) * n, s) != cudaSuccess)
        return HL_OUT_OF_MEM;
    if (cudaMallocAsync(&dd, sizeof(hl_image_desc) * n, s) != cudaSuccess) {
        cudaFreeAsync(dp, s);
        return HL_OUT_OF_MEM;
    }
    cudaError_t e = cudaMemcpyAsync(dp, params, sizeof(hl_scene_params) * n,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dd, outs, sizeof(hl_image_desc) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        hl_synth_kernel<<<n, 256, 0, s>>>(dp, dd);
        e = cudaGetLastError();
    }
    cudaFreeAsync(dp, s);
    cudaFreeAsync(dd, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? HL_NO_ERROR : HL_CUDA_ERROR;
}
