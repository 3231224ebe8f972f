// houghline_class_main.cpp -- exercises the drop-in C++ surface
// (include/HoughLine.h, Image.h, CoordiSet.h) the way a caller of the
// reference would, and prints every result in an exact text form (floats as
// hex) for tests/test_cpp_class.py to compare against the oracle.
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "CoordiSet.h"
#include "HoughLine.h"
#include "Image.h"
#include "houghline_gb300.h"

static uint64_t fnv(const unsigned char *p, size_t n)
{
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; i++) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

static void print_lines(const char *tag, int rc, int n, const LineParam *l)
{
    printf("%s rc=%d n=%d\n", tag, rc, n);
    for (int i = 0; i < n; i++)
        printf("%s line %a %d %d\n", tag, l[i].angle, l[i].distance, l[i].votes);
}

int main(int argc, char **argv)
{
    const int W = 512, H = 512;
    // the 512 x 512 scene of the single-image workload, seed 1234
    hl_scene_params sp[1];
    hl_synth_spec(1, 1234, 1, sp);

    Image *img = NULL;
    ImageBasicOp::newImage(&img);
    ImageBasicOp::makeAtHost(img, W, H);
    hl_synth_scene(&sp[0], img->imgData, W);
    printf("image fnv=%llu\n", (unsigned long long)fnv(img->imgData, (size_t)W * H));

    HoughLine hough(M_PI / 180, 1.0, 100, (float)(M_PI / 180 * 5.0), 50);
    LineParam lines[16];
    int lm = 16;
    int rc = hough.houghLine(img, NULL, &lm, lines);
    print_lines("plain", rc, lm, lines);
    // the reference migrates the input image to the current device in place
    printf("migrated deviceId=%d pitch_ok=%d\n", IMAGE_CUDA(img)->deviceId,
           (int)(IMAGE_CUDA(img)->pitchBytes >= (size_t)W));

    // ROI + getGlobalParam
    img->roiX1 = 37;
    img->roiY1 = 21;
    img->roiX2 = 480;
    img->roiY2 = 500;
    lm = 16;
    rc = hough.houghLine(img, NULL, &lm, lines);
    print_lines("roi", rc, lm, lines);
    rc = hough.getGlobalParam(img, &lm, lines);
    print_lines("global", rc, lm, lines);
    img->roiX1 = img->roiY1 = 0;
    img->roiX2 = W;
    img->roiY2 = H;

    // houghLineImg into an empty output image (created with the ROI's size)
    Image *out = NULL;
    ImageBasicOp::newImage(&out);
    lm = 16;
    rc = hough.houghLineImg(img, NULL, out, &lm, lines);
    print_lines("img", rc, lm, lines);
    ImageBasicOp::copyToHost(out);
    size_t lit = 0;
    for (size_t i = 0; i < out->width * out->height; i++)
        lit += out->imgData[i] == 255;
    printf("drawn %zux%zu fnv=%llu lit=%zu\n", out->width, out->height,
           (unsigned long long)fnv(out->imgData, out->width * out->height), lit);

    // realLine on a few segments (tests/test_cpp_class.py recomputes them)
    const int segs[4][4] = {{0, 0, 511, 511}, {100, 50, 400, 50},
                            {17, 300, 480, 120}, {5, 5, 5, 400}};
    for (int i = 0; i < 4; i++)
        printf("realline %d %d\n", i,
               (int)hough.realLine(img, segs[i][0], segs[i][1], segs[i][2],
                                   segs[i][3], 2.5f, 0.05f));

    // coordinate-set path: the image's edge pixels as a CoordiSet
    ImageBasicOp::copyToHost(img);
    size_t n = 0;
    for (size_t i = 0; i < (size_t)W * H; i++)
        n += img->imgData[i] == 255;
    CoordiSet *cst = NULL;
    CoordiSetBasicOp::newCoordiSet(&cst);
    CoordiSetBasicOp::makeAtHost(cst, n);
    size_t k = 0;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            if (img->imgData[(size_t)y * W + x] == 255) {
                cst->tplData[2 * k] = x;
                cst->tplData[2 * k + 1] = y;
                k++;
            }
    lm = 16;
    rc = hough.houghLine(NULL, cst, &lm, lines);
    print_lines("points", rc, lm, lines);

    // argument checks
    printf("null=%d\n", hough.houghLine(NULL, NULL, &lm, lines));
    CoordiSetBasicOp::deleteCoordiSet(cst);
    ImageBasicOp::deleteImage(out);
    ImageBasicOp::deleteImage(img);
    (void)argc;
    (void)argv;
    return 0;
}
