/* hl_synth.h -- seeded synthetic edge scenes (see synth.c). */
#ifndef HL_SYNTH_H
#define HL_SYNTH_H

#include "houghline_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
    HL_SPEC_PLAIN_512 = 1,     /* one 512x512 image */
    HL_SPEC_PLAIN_4096 = 2,    /* one 4096x4096 image */
    HL_SPEC_BATCH_UNEVEN = 3,  /* uneven 256..2048 images */
    HL_SPEC_PROPOSAL_2048 = 4, /* 2048x2048 proposal-training images */
    HL_SPEC_MIXED_UNEVEN = 5   /* uneven 512..4096, sparse / cluttered mix */
};

/* Integer Bresenham segment, clipped to the image. */
void hl_synth_bresenham(uint8_t *img, long pitch, int w, int h,
                        int x0, int y0, int x1, int y1);

#ifdef __cplusplus
}
#endif
#endif
