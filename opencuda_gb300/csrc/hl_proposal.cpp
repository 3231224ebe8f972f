/*
 * hl_proposal.cpp -- the C ABI of the proposal network: single-layer entry
 * points (used by the parity tests), the network object (forward, training
 * step with the project's own backward kernels and Adam) and the
 * proposal-guided HoughLine pipeline.
 */
#include <cuda_runtime.h>

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "hl_cnn.h"
#include "hl_internal.h"

static int cnn_err(cudaError_t e)
{
    if (e == cudaSuccess)
        return HL_NO_ERROR;
    return e == cudaErrorMemoryAllocation ? HL_OUT_OF_MEM : HL_CUDA_ERROR;
}

#define CKN(call)                                 \
    do {                                          \
        cudaError_t e__ = (call);                 \
        if (e__ != cudaSuccess)                   \
            return cnn_err(e__);                  \
    } while (0)

extern "C" int hl_cnn_conv3x3(const void *x, const void *w, const float *bias,
                              void *y, float *y_f32, int B, int H, int W,
                              int cin, int cout, int stride, int relu,
                              int mode, int *status_dev, void *stream)
{
    if (!x || !w || (!y && !y_f32) || !status_dev)
        return HL_NULL_POINTER;
    if (B <= 0 || H <= 0 || W <= 0 || (cin != 1 && cin != 32) || cout < 1 ||
        cout > 32 || (stride != 1 && stride != 2) || (mode != 0 && mode != 1))
        return HL_INVALID_DATA;
    if ((y_f32 && cout != 1) || (mode == 1 && (stride != 2 || cin != 32)))
        return HL_INVALID_DATA;
    hl_conv_args a;
    memset(&a, 0, sizeof(a));
    a.x = static_cast<const __nv_bfloat16 *>(x);
    a.w = static_cast<const __nv_bfloat16 *>(w);
    a.bias = bias;
    a.y = static_cast<__nv_bfloat16 *>(y);
    a.y_f32 = y_f32;
    a.B = B;
    a.H = H;
    a.W = W;
    if (mode == 0) {
        a.Ho = (H - 1) / stride + 1;
        a.Wo = (W - 1) / stride + 1;
    } else {   /* x-gradient of a stride-2 conv whose input was 2H x 2W */
        a.Ho = 2 * H;
        a.Wo = 2 * W;
    }
    a.cin = cin;
    a.cout = cout;
    a.kreal = 9 * cin;
    a.stride = stride;
    a.relu = relu;
    a.status = status_dev;
    CKN(hl_launch_conv3x3(&a, mode, reinterpret_cast<cudaStream_t>(stream)));
    return HL_NO_ERROR;
}
