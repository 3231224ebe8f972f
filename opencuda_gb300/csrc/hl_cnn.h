/*
 * hl_cnn.h -- kernel argument blocks and launchers of the proposal network
 * (not part of the C ABI).
 */
#ifndef HL_CNN_H
#define HL_CNN_H

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

/* 3x3 convolution, padding 1: x [B][H][W][cin] -> y [B][Ho][Wo][cout] */
typedef struct hl_conv_args {
    const __nv_bfloat16 *x;
    const __nv_bfloat16 *w;   /* [cout][kreal], kreal = 9 * cin */
    const float *bias;        /* [cout] or NULL */
    __nv_bfloat16 *y;         /* bf16 NHWC with 32 channels ... */
    float *y_f32;             /* ... or f32 [B][Ho][Wo] when cout == 1 */
    int B, H, W, Ho, Wo;
    int cin, cout, kreal;
    int stride;
    int relu;
    int *status;
} hl_conv_args;

/* mode 0: convolution; mode 1: input gradient of a stride-2 convolution
 * (x = dy, w = the transposed weights [cin][9 * cout], Ho x Wo = the input
 * size of the forward convolution) */
cudaError_t hl_launch_conv3x3(const hl_conv_args *a, int mode, cudaStream_t s);

#endif
