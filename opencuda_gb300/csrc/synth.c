/*
 * synth.c -- seeded synthetic binary edge scenes (0/255 uint8) for the
 * HoughLine workloads: Bresenham segments, quadratic Bezier curves and
 * uniform salt noise.
 *
 * Integer arithmetic only, so one seed gives the same image on every host
 * (x86-64 build machine, aarch64 Grace GPU host).  The reference ships no
 * generator and no test images; these scenes stand in for its edge-detector
 * outputs (okano_3_0/RobustEdgeDetection.cu and friends produce 0/255 maps of
 * the same form).
 */
#include "hl_synth.h"

#include <string.h>

static inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline uint64_t next64(uint64_t *s)
{
    *s += 0x9E3779B97F4A7C15ull;
    return mix64(*s);
}

/* uniform integer in [lo, hi] (inclusive), Lemire's multiply-shift */
static inline int64_t urange(uint64_t *s, int64_t lo, int64_t hi)
{
    if (hi <= lo)
        return lo;
    uint64_t span = (uint64_t)(hi - lo) + 1u;
    unsigned __int128 m = (unsigned __int128)next64(s) * span;
    return lo + (int64_t)(uint64_t)(m >> 64);
}

static inline void plot(uint8_t *img, long pitch, int w, int h, int x, int y)
{
    if (x >= 0 && y >= 0 && x < w && y < h)
        img[(long)y * pitch + x] = 255;
}

void hl_synth_bresenham(uint8_t *img, long pitch, int w, int h,
                        int x0, int y0, int x1, int y1)
{
    int dx = x1 > x0 ? x1 - x0 : x0 - x1;
    int dy = y1 > y0 ? y0 - y1 : y1 - y0;   /* -|dy| */
    int sx = x0 < x1 ? 1 : -1;
    int sy = y0 < y1 ? 1 : -1;
    int err = dx + dy;
    for (;;) {
        plot(img, pitch, w, h, x0, y0);
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

static void draw_bezier(uint8_t *img, long pitch, int w, int h, uint64_t *s)
{
    int64_t px[3], py[3];
    for (int i = 0; i < 3; i++) {
        px[i] = urange(s, 0, w - 1);
        py[i] = urange(s, 0, h - 1);
    }
    int64_t n = (px[1] > px[0] ? px[1] - px[0] : px[0] - px[1]) +
                (py[1] > py[0] ? py[1] - py[0] : py[0] - py[1]) +
                (px[2] > px[1] ? px[2] - px[1] : px[1] - px[2]) +
                (py[2] > py[1] ? py[2] - py[1] : py[1] - py[2]);
    if (n < 1)
        n = 1;
    int64_t n2 = n * n;
    int lx = (int)px[0], ly = (int)py[0];
    for (int64_t i = 1; i <= n; i++) {
        int64_t a = (n - i) * (n - i), b = 2 * (n - i) * i, c = i * i;
        int x = (int)((a * px[0] + b * px[1] + c * px[2] + n2 / 2) / n2);
        int y = (int)((a * py[0] + b * py[1] + c * py[2] + n2 / 2) / n2);
        hl_synth_bresenham(img, pitch, w, h, lx, ly, x, y);
        lx = x;
        ly = y;
    }
}

int hl_synth_scene(const hl_scene_params *p, uint8_t *img, long pitch)
{
    if (!p || !img || p->width <= 0 || p->height <= 0 || pitch < p->width)
        return -1;
    int w = p->width, h = p->height;
    for (int y = 0; y < h; y++)
        memset(img + (long)y * pitch, 0, (size_t)w);
    uint64_t s = p->seed * 0xD1342543DE82EF95ull + 0x1234567ull;
    int64_t lmin = p->len_min, lmax = p->len_max;
    if (lmax < lmin)
        lmax = lmin;
    int64_t lmin2 = lmin * lmin, lmax2 = lmax * lmax;
    for (int i = 0; i < p->nseg; i++) {
        /* start uniform in the image; offset uniform in the square
         * [-lmax, lmax]^2, kept when its length lies in [lmin, lmax] and
         * the far end lies inside the image (bounded retries) */
        int x0 = 0, y0 = 0, x1 = 0, y1 = 0, ok = 0;
        for (int attempt = 0; attempt < 64 && !ok; attempt++) {
            x0 = (int)urange(&s, 0, w - 1);
            y0 = (int)urange(&s, 0, h - 1);
            for (int t = 0; t < 256; t++) {
                int64_t dx = urange(&s, -lmax, lmax);
                int64_t dy = urange(&s, -lmax, lmax);
                int64_t l2 = dx * dx + dy * dy;
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
        if (ok)
            hl_synth_bresenham(img, pitch, w, h, x0, y0, x1, y1);
    }
    for (int i = 0; i < p->nbezier; i++)
        draw_bezier(img, pitch, w, h, &s);
    if (p->salt_ppm > 0) {
        uint64_t key = mix64(p->seed ^ 0x5A17C0DEull);
        for (int y = 0; y < h; y++) {
            uint8_t *row = img + (long)y * pitch;
            uint64_t base = key + (uint64_t)y * (uint64_t)w * 0x9E3779B97F4A7C15ull;
            for (int x = 0; x < w; x++) {
                uint64_t r = mix64(base + (uint64_t)x * 0x9E3779B97F4A7C15ull);
                if ((r % 1000000u) < (uint64_t)p->salt_ppm)
                    row[x] = 255;
            }
        }
    }
    return 0;
}

/* Workload specs.  Each draws the per-image parameters from one seeded
 * stream so a (kind, seed, index) triple names an image everywhere. */
int hl_synth_spec(int kind, uint64_t seed, int n, hl_scene_params *out)
{
    if (!out || n < 0)
        return -1;
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + (uint64_t)kind;
    for (int i = 0; i < n; i++) {
        hl_scene_params *p = &out[i];
        memset(p, 0, sizeof(*p));
        p->seed = seed * 1000003ull + (uint64_t)i;
        switch (kind) {
        case HL_SPEC_PLAIN_512:      /* 512^2, 8 segments 100-400 px, 1% salt */
            p->width = p->height = 512;
            p->nseg = 8;
            p->len_min = 100;
            p->len_max = 400;
            p->salt_ppm = 10000;
            break;
        case HL_SPEC_PLAIN_4096:     /* 4096^2, 64 segments 200-3000 px, 2% salt */
            p->width = p->height = 4096;
            p->nseg = 64;
            p->len_min = 200;
            p->len_max = 3000;
            p->salt_ppm = 20000;
            break;
        case HL_SPEC_BATCH_UNEVEN: { /* w,h in [256,2048], 4-32 segs, 0.5-3% salt */
            p->width = (int)urange(&s, 256, 2048);
            p->height = (int)urange(&s, 256, 2048);
            p->nseg = (int)urange(&s, 4, 32);
            p->salt_ppm = (int)urange(&s, 5000, 30000);
            /* segment length U[0.1, 1.0] * diagonal (integer sqrt) */
            int64_t d2 = (int64_t)p->width * p->width + (int64_t)p->height * p->height;
            int64_t d = 0;
            while ((d + 1) * (d + 1) <= d2)
                d++;
            p->len_min = (int)(d / 10);
            p->len_max = (int)d;
            break;
        }
        case HL_SPEC_PROPOSAL_2048: /* 2048^2, 8-48 segs, 1-4% noise */
            p->width = p->height = 2048;
            p->nseg = (int)urange(&s, 8, 48);
            p->salt_ppm = (int)urange(&s, 10000, 40000);
            p->len_min = 200;
            p->len_max = 2048;
            break;
        case HL_SPEC_MIXED_UNEVEN: { /* 70% sparse / 30% cluttered, w,h in [512,4096] */
            p->width = (int)urange(&s, 512, 4096);
            p->height = (int)urange(&s, 512, 4096);
            int cluttered = urange(&s, 0, 99) < 30;
            if (cluttered) {
                p->nseg = (int)urange(&s, 64, 128);
                p->nbezier = 20;
                p->salt_ppm = 80000;
            } else {
                p->nseg = (int)urange(&s, 4, 32);
                p->salt_ppm = 10000;
            }
            int64_t d2 = (int64_t)p->width * p->width + (int64_t)p->height * p->height;
            int64_t d = 0;
            while ((d + 1) * (d + 1) <= d2)
                d++;
            p->len_min = (int)(d / 10);
            p->len_max = (int)d;
            break;
        }
        default:
            return -1;
        }
    }
    return 0;
}
