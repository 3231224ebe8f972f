/*
 * hl_cnn.h -- kernel argument blocks and launchers of the proposal network
 * (not part of the C ABI).
 */
#ifndef HL_CNN_H
#define HL_CNN_H

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

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

/* Weight gradient of a 3x3 convolution (padding 1): dw [cout][9 * cin] +=,
 * db [cout] += (NULL: none).  x as in the forward pass, dy [P][dy_c] f32
 * (dy_c = 32, or 1 for a one-channel output). */
typedef struct hl_dw_args {
    const __nv_bfloat16 *x;
    const float *dy;          /* [P][dy_c] */
    int dy_c;
    float *dw;
    float *db;
    int B, H, W, Ho, Wo;
    int cin, cout;
    int stride;
} hl_dw_args;
cudaError_t hl_launch_conv_dw(const hl_dw_args *a, cudaStream_t s);

cudaError_t hl_launch_relu_mask(const __nv_bfloat16 *dx, const __nv_bfloat16 *y,
                                long long n, float *out_f32,
                                __nv_bfloat16 *out_bf16, cudaStream_t s);

/* Average pooling of 0/255 images into side x side occupancy maps. */
typedef struct hl_pool_img {
    const uint8_t *base;   /* ROI origin */
    long pitch;
    int w, h;
    int factor;            /* pooled cell = factor x factor pixels */
    int pad;
} hl_pool_img;
cudaError_t hl_launch_pool(const hl_pool_img *imgs, int nimg, int side,
                           __nv_bfloat16 *out, cudaStream_t s);

/* The fixed coarse Hough head: HL_HEAD_T angles (cell centres of
 * 180 / HL_HEAD_T degrees) x HL_HEAD_R rho bins over the image's rho range. */
#define HL_HEAD_T 90
#define HL_HEAD_R 128
typedef struct hl_head_geom {
    float cell;      /* evidence cell size in image pixels */
    float rho_min;   /* the image's rho range start */
    float inv_rw;    /* coarse bins per rho unit: 128 / R */
    int qh, qw;      /* evidence cells covering the ROI */
    int pad;
} hl_head_geom;
cudaError_t hl_launch_head_fwd(const float *e, int ev, const hl_head_geom *geo,
                               int nimg, const float *ab, float *hsum,
                               float *logits, cudaStream_t s);
cudaError_t hl_launch_head_bwd(const float *dz, int ev, const hl_head_geom *geo,
                               int nimg, const float *ab, float *de, cudaStream_t s);
cudaError_t hl_launch_bce(const float *z, const float *y, const float *hsum,
                          long long n, float wpos, float *dz, float *dab,
                          float *loss, cudaStream_t s);
cudaError_t hl_launch_adam(float *w, const float *g, float *m, float *v, int n,
                           float lr, int step, float clip, cudaStream_t s);
cudaError_t hl_launch_f32_to_bf16(const float *in, long long n, __nv_bfloat16 *out,
                                  cudaStream_t s);
cudaError_t hl_launch_weight_layout(const float *w, int cout, int cin, int mode,
                                    __nv_bfloat16 *out, cudaStream_t s);

struct hl_net;
/* the network's forward pass on device-resident geometry (hl_proposal.cpp);
 * *logits points into the network's own buffer */
int hl_net_run(struct hl_net *n, const __nv_bfloat16 *occ,
               const hl_head_geom *geo_dev, int B, const float **logits,
               cudaStream_t s);
/* stream-ordered copy of the network's status word into *st (pinned) */
int hl_net_status(struct hl_net *n, int *st, cudaStream_t s);

#endif
