// houghcircle_class_main.cpp -- exercises the drop-in C++ HoughCircle class
// (include/HoughCircle.h) the way a caller of the reference would, on a raw
// w x h image read from argv[1], and prints every result for
// tests/test_cpp_class.py to compare against the oracle.
#include <stdio.h>
#include <stdlib.h>

#include "CoordiSet.h"
#include "HoughCircle.h"
#include "Image.h"

static void print_circles(const char *tag, int rc, int n, const CircleParam *c)
{
    printf("%s rc=%d n=%d\n", tag, rc, n);
    for (int i = 0; i < n; i++)
        printf("%s circle %d %d %d %d\n", tag, c[i].a, c[i].b, c[i].radius, c[i].votes);
}

int main(int argc, char **argv)
{
    if (argc < 4)
        return 2;
    const int W = atoi(argv[2]), H = atoi(argv[3]);
    Image *img = NULL;
    ImageBasicOp::newImage(&img);
    ImageBasicOp::makeAtHost(img, W, H);
    FILE *f = fopen(argv[1], "rb");
    if (!f || fread(img->imgData, 1, (size_t)W * H, f) != (size_t)W * H)
        return 3;
    fclose(f);

    HoughCircle hc(5, 50, 30.0f, 10, 60);
    CircleParam cir[64];
    int cm = 32;
    int rc = hc.houghcircle(img, NULL, &cm, cir, false);
    print_circles("full", rc, cm, cir);

    img->roiX1 = 40;
    img->roiY1 = 30;
    img->roiX2 = W - 20;
    img->roiY2 = H - 10;
    cm = 32;
    rc = hc.houghcircle(img, NULL, &cm, cir, false);
    print_circles("roi", rc, cm, cir);
    img->roiX1 = img->roiY1 = 0;
    img->roiX2 = W;
    img->roiY2 = H;

    cm = 64;
    rc = hc.pieceCircle(img, 2, &cm, cir, false);
    print_circles("piece", rc, cm, cir);
    printf("lastroi %d %d %d %d\n", img->roiX1, img->roiY1, img->roiX2, img->roiY2);

    // coordinate-set path: the image's edge pixels
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
    cm = 32;
    rc = hc.houghcircle(NULL, cst, &cm, cir, false);
    print_circles("points", rc, cm, cir);

    // pieceCircle with one piece that overflows the candidate buffer (argv[4]:
    // a second W x H image whose bottom-right piece is dense noise): the
    // other pieces' circles are kept, as the reference keeps them
    if (argc > 4) {
        Image *ov = NULL;
        ImageBasicOp::newImage(&ov);
        ImageBasicOp::makeAtHost(ov, W, H);
        FILE *g = fopen(argv[4], "rb");
        if (!g || fread(ov->imgData, 1, (size_t)W * H, g) != (size_t)W * H)
            return 4;
        fclose(g);
        ov->roiX1 = W / 2;
        ov->roiY1 = H / 2;
        ov->roiX2 = W / 2 + W / 2 - 1;
        ov->roiY2 = H / 2 + H / 2 - 1;
        cm = 32;
        printf("ovrc=%d\n", hc.houghcircle(ov, NULL, &cm, cir, false));
        ov->roiX1 = ov->roiY1 = 0;
        ov->roiX2 = W;
        ov->roiY2 = H;
        cm = 64;
        rc = hc.pieceCircle(ov, 2, &cm, cir, false);
        print_circles("pieceov", rc, cm, cir);
        ImageBasicOp::deleteImage(ov);
    }

    // argument checks and the setters' validation
    printf("null=%d\n", hc.houghcircle(NULL, NULL, &cm, cir, false));
    HoughCircle d;
    printf("defaults %d %d %d %d %d\n", d.getRadiusMin(), d.getRadiusMax(),
           (int)d.getDistThres(), d.getRThres(), d.getCirThreshold());
    printf("setmin=%d keep=%d\n", d.setRadiusMin(-1), d.getRadiusMin());
    printf("setthr=%d keep=%d\n", d.setCirThreshold(-5), d.getCirThreshold());
    CoordiSetBasicOp::deleteCoordiSet(cst);
    ImageBasicOp::deleteImage(img);
    return 0;
}
