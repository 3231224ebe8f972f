/*
 * hl_proposal.h -- C ABI of the learned proposal stage: a small CNN
 * (six 3x3 convolutions, 32 channels, BF16 weights and activations, FP32
 * accumulation on the tensor cores) reads an average-pooled edge map and
 * scores coarse (theta, rho) cells; the exact int32 vote then runs only in
 * the best cells.  No counterpart in the reference (its HoughLine always
 * votes the full accumulator, okano_3_0/HoughLine.cu:635-955); every line
 * it reports carries the exact vote count the full method gives that bin.
 *
 * Device pointers throughout; every call returns an hl ErrorCode.
 */
#ifndef HL_PROPOSAL_H
#define HL_PROPOSAL_H

#include "houghline_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One 3x3 convolution with padding 1 (the network's building block, exposed
 * for parity tests).  x: [B][H][W][cin] bf16 (cin = 1 or 32); w: [cout][9 *
 * cin] bf16 (k = (ky * 3 + kx) * cin + ci); bias: [cout] f32 or NULL.  Output
 * y: [B][Ho][Wo][32] bf16 (channels >= cout written as 0), or y_f32:
 * [B][Ho][Wo] f32 when cout = 1.  mode 0: convolution with the given stride,
 * Ho = (H - 1) / stride + 1; mode 1: input gradient of a stride-2
 * convolution: x = the output gradient (cin = 32), w = the transposed
 * weights [cin_fwd][9 * 32] with w'[ci][tap][co] = w[co][tap][ci], output
 * 2H x 2W.  relu: apply max(0, .) in the epilogue.  In-kernel time-outs set
 * bit 0x20 of *status_dev. */
int hl_cnn_conv3x3(const void *x, const void *w, const float *bias, void *y,
                   float *y_f32, int B, int H, int W, int cin, int cout,
                   int stride, int relu, int mode, int *status_dev,
                   void *stream);

#ifdef __cplusplus
}
#endif
#endif
