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
#include "hl_proposal.h"

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

/* ==================================================================== */
/* The network                                                           */
/* ==================================================================== */

/* Layers: (cin, cout, stride, relu); input 256 x 256 x 1, evidence 64 x 64. */
#define NET_LAYERS 6
static const int L_CIN[NET_LAYERS] = {1, 32, 32, 32, 32, 32};
static const int L_COUT[NET_LAYERS] = {32, 32, 32, 32, 32, 1};
static const int L_STRIDE[NET_LAYERS] = {2, 2, 1, 1, 1, 1};
static const int L_RELU[NET_LAYERS] = {1, 1, 1, 1, 1, 0};
#define NET_IN 256
#define NET_EV 64

/* flat FP32 parameter offsets: per layer W [cout][9 cin] then b [cout]; then
 * the head's alpha, beta */
static int w_off(int l)
{
    int o = 0;
    for (int i = 0; i < l; i++)
        o += L_COUT[i] * 9 * L_CIN[i] + L_COUT[i];
    return o;
}
static int b_off(int l) { return w_off(l) + L_COUT[l] * 9 * L_CIN[l]; }
static int ab_off(void) { return w_off(NET_LAYERS); }
static int n_params(void) { return ab_off() + 2; }

/* side of layer l's input and output */
static int l_in_side(int l) { return l == 0 ? NET_IN : (l == 1 ? NET_IN / 2 : NET_EV); }
static int l_out_side(int l) { return l == 0 ? NET_IN / 2 : NET_EV; }

struct hl_net {
    int B;                             /* capacity (images) */
    float *w, *g, *m, *v;              /* FP32 master weights, grads, Adam */
    __nv_bfloat16 *wf[NET_LAYERS];     /* forward bf16 weights */
    __nv_bfloat16 *wb[NET_LAYERS];     /* backward layouts (l >= 1) */
    __nv_bfloat16 *act[NET_LAYERS];    /* outputs of layers 0..4 (bf16) */
    float *ev;                         /* layer 5 output, [B][64][64] */
    float *hsum, *logits, *dz;         /* [B][90][128] */
    float *de;                         /* [B][64][64] */
    __nv_bfloat16 *de_b;
    __nv_bfloat16 *gx, *gx2;           /* input gradients (bf16, 32 ch) */
    float *gm;                         /* masked gradient f32 [P][32] */
    __nv_bfloat16 *gm_b;
    float *loss;                       /* [1] */
    int *status;
    hl_head_geom *geo;                 /* [B] */
    int step;
};

static void net_free_bufs(hl_net *n)
{
    void *p[] = {n->ev, n->hsum, n->logits, n->dz, n->de, n->de_b, n->gx, n->gx2,
                 n->gm, n->gm_b, n->geo};
    for (void *q : p)
        if (q)
            cudaFree(q);
    for (int l = 0; l < NET_LAYERS; l++)
        if (n->act[l])
            cudaFree(n->act[l]);
    n->ev = n->hsum = n->logits = n->dz = n->de = n->gm = nullptr;
    n->de_b = n->gx = n->gx2 = n->gm_b = nullptr;
    n->geo = nullptr;
    for (int l = 0; l < NET_LAYERS; l++)
        n->act[l] = nullptr;
    n->B = 0;
}

static int net_reserve(hl_net *n, int B)
{
    if (B <= n->B)
        return HL_NO_ERROR;
    net_free_bufs(n);
    const size_t s128 = (size_t)B * 128 * 128, s64 = (size_t)B * 64 * 64;
    const size_t cells = (size_t)B * HL_HEAD_T * HL_HEAD_R;
    CKN(cudaMalloc(&n->act[0], s128 * 32 * sizeof(__nv_bfloat16)));
    for (int l = 1; l < 5; l++)
        CKN(cudaMalloc(&n->act[l], s64 * 32 * sizeof(__nv_bfloat16)));
    CKN(cudaMalloc(&n->ev, s64 * sizeof(float)));
    CKN(cudaMalloc(&n->hsum, cells * sizeof(float)));
    CKN(cudaMalloc(&n->logits, cells * sizeof(float)));
    CKN(cudaMalloc(&n->dz, cells * sizeof(float)));
    CKN(cudaMalloc(&n->de, s64 * sizeof(float)));
    CKN(cudaMalloc(&n->de_b, s64 * sizeof(__nv_bfloat16)));
    CKN(cudaMalloc(&n->gx, s128 * 32 * sizeof(__nv_bfloat16)));
    CKN(cudaMalloc(&n->gx2, s128 * 32 * sizeof(__nv_bfloat16)));
    CKN(cudaMalloc(&n->gm, s128 * 32 * sizeof(float)));
    CKN(cudaMalloc(&n->gm_b, s128 * 32 * sizeof(__nv_bfloat16)));
    CKN(cudaMalloc(&n->geo, (size_t)B * sizeof(hl_head_geom)));
    n->B = B;
    return HL_NO_ERROR;
}

/* bf16 copies of the master weights in every layout the passes use */
static int net_refresh(hl_net *n, cudaStream_t s)
{
    for (int l = 0; l < NET_LAYERS; l++) {
        CKN(hl_launch_weight_layout(n->w + w_off(l), L_COUT[l], L_CIN[l], 0, n->wf[l], s));
        if (l >= 1)
            CKN(hl_launch_weight_layout(n->w + w_off(l), L_COUT[l], L_CIN[l],
                                        L_STRIDE[l] == 1 ? 1 : 2, n->wb[l], s));
    }
    return HL_NO_ERROR;
}

/* deterministic He-style initialisation (splitmix64 -> Box-Muller) */
static uint64_t sm64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

extern "C" int hl_net_num_params(void) { return n_params(); }

extern "C" int hl_net_create(hl_net **out, unsigned long long seed)
{
    if (!out)
        return HL_NULL_POINTER;
    *out = nullptr;
    hl_net *n = new (std::nothrow) hl_net();
    if (!n)
        return HL_OUT_OF_MEM;
    memset(n, 0, sizeof(*n));
    const int np = n_params();
    int rc = HL_NO_ERROR;
    auto fail = [&](int r) { hl_net_destroy(n); return r; };
    if (cudaMalloc(&n->w, np * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&n->g, np * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&n->m, np * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&n->v, np * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&n->loss, sizeof(float)) != cudaSuccess ||
        cudaMalloc(&n->status, sizeof(int)) != cudaSuccess)
        return fail(HL_OUT_OF_MEM);
    for (int l = 0; l < NET_LAYERS; l++) {
        const size_t k = (size_t)L_COUT[l] * 9 * L_CIN[l];
        if (cudaMalloc(&n->wf[l], k * sizeof(__nv_bfloat16)) != cudaSuccess ||
            cudaMalloc(&n->wb[l], k * sizeof(__nv_bfloat16)) != cudaSuccess)
            return fail(HL_OUT_OF_MEM);
    }
    std::vector<float> h((size_t)np, 0.0f);
    uint64_t st = seed ^ 0x6A09E667F3BCC909ull;
    for (int l = 0; l < NET_LAYERS; l++) {
        const int fan = 9 * L_CIN[l];
        const float sd = sqrtf(2.0f / (float)fan);
        for (int i = 0; i < L_COUT[l] * fan; i++) {
            double u1 = ((double)(sm64(&st) >> 11) + 0.5) / 9007199254740992.0;
            double u2 = ((double)(sm64(&st) >> 11) + 0.5) / 9007199254740992.0;
            h[(size_t)w_off(l) + i] =
                (float)(sd * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
        }
    }
    h[(size_t)ab_off()] = 1.0f;    /* alpha */
    h[(size_t)ab_off() + 1] = -4.0f;   /* beta: lines are rare */
    if (cudaMemcpy(n->w, h.data(), np * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(n->m, 0, np * sizeof(float)) != cudaSuccess ||
        cudaMemset(n->v, 0, np * sizeof(float)) != cudaSuccess ||
        cudaMemset(n->status, 0, sizeof(int)) != cudaSuccess)
        return fail(HL_CUDA_ERROR);
    if ((rc = net_refresh(n, 0)) != HL_NO_ERROR || cudaStreamSynchronize(0) != cudaSuccess)
        return fail(rc != HL_NO_ERROR ? rc : HL_CUDA_ERROR);
    *out = n;
    return HL_NO_ERROR;
}

extern "C" int hl_net_destroy(hl_net *n)
{
    if (!n)
        return HL_NULL_POINTER;
    net_free_bufs(n);
    void *p[] = {n->w, n->g, n->m, n->v, n->loss, n->status};
    for (void *q : p)
        if (q)
            cudaFree(q);
    for (int l = 0; l < NET_LAYERS; l++) {
        if (n->wf[l])
            cudaFree(n->wf[l]);
        if (n->wb[l])
            cudaFree(n->wb[l]);
    }
    delete n;
    return HL_NO_ERROR;
}

extern "C" int hl_net_get_params(hl_net *n, float *host)
{
    if (!n || !host)
        return HL_NULL_POINTER;
    CKN(cudaMemcpy(host, n->w, n_params() * sizeof(float), cudaMemcpyDeviceToHost));
    return HL_NO_ERROR;
}

extern "C" int hl_net_get_grads(hl_net *n, float *host)
{
    if (!n || !host)
        return HL_NULL_POINTER;
    CKN(cudaMemcpy(host, n->g, n_params() * sizeof(float), cudaMemcpyDeviceToHost));
    return HL_NO_ERROR;
}

extern "C" int hl_net_set_params(hl_net *n, const float *host)
{
    if (!n || !host)
        return HL_NULL_POINTER;
    CKN(cudaMemcpy(n->w, host, n_params() * sizeof(float), cudaMemcpyHostToDevice));
    CKN(cudaMemset(n->m, 0, n_params() * sizeof(float)));
    CKN(cudaMemset(n->v, 0, n_params() * sizeof(float)));
    n->step = 0;
    int rc = net_refresh(n, 0);
    if (rc != HL_NO_ERROR)
        return rc;
    CKN(cudaStreamSynchronize(0));
    return HL_NO_ERROR;
}

static int conv_layer(hl_net *n, int l, const __nv_bfloat16 *x, int B,
                      __nv_bfloat16 *y, float *y_f32, cudaStream_t s)
{
    hl_conv_args a;
    memset(&a, 0, sizeof(a));
    a.x = x;
    a.w = n->wf[l];
    a.bias = n->w + b_off(l);
    a.y = y;
    a.y_f32 = y_f32;
    a.B = B;
    a.H = a.W = l_in_side(l);
    a.Ho = a.Wo = l_out_side(l);
    a.cin = L_CIN[l];
    a.cout = L_COUT[l];
    a.kreal = 9 * L_CIN[l];
    a.stride = L_STRIDE[l];
    a.relu = L_RELU[l];
    a.status = n->status;
    CKN(hl_launch_conv3x3(&a, 0, s));
    return HL_NO_ERROR;
}

static int net_forward(hl_net *n, const __nv_bfloat16 *occ, int B, cudaStream_t s)
{
    int rc;
    const __nv_bfloat16 *x = occ;
    for (int l = 0; l < NET_LAYERS; l++) {
        if (l < NET_LAYERS - 1)
            rc = conv_layer(n, l, x, B, n->act[l], nullptr, s);
        else
            rc = conv_layer(n, l, x, B, nullptr, n->ev, s);
        if (rc != HL_NO_ERROR)
            return rc;
        x = n->act[l];
    }
    CKN(hl_launch_head_fwd(n->ev, NET_EV, n->geo, B, n->w + ab_off(), n->hsum,
                           n->logits, s));
    return HL_NO_ERROR;
}

static int upload_geo(hl_net *n, const hl_coarse_geom *geo, int B, cudaStream_t s)
{
    static_assert(sizeof(hl_coarse_geom) == sizeof(hl_head_geom), "geometry layout");
    CKN(cudaMemcpyAsync(n->geo, geo, (size_t)B * sizeof(hl_head_geom),
                        cudaMemcpyHostToDevice, s));
    return HL_NO_ERROR;
}

extern "C" int hl_net_forward(hl_net *n, const void *occ_dev,
                              const hl_coarse_geom *geo_host, int B,
                              float *logits_dev, void *stream)
{
    if (!n || !occ_dev || !geo_host || !logits_dev)
        return HL_NULL_POINTER;
    if (B <= 0)
        return HL_INVALID_DATA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int rc = net_reserve(n, B);
    if (rc != HL_NO_ERROR || (rc = upload_geo(n, geo_host, B, s)) != HL_NO_ERROR)
        return rc;
    if ((rc = net_forward(n, static_cast<const __nv_bfloat16 *>(occ_dev), B, s)) !=
        HL_NO_ERROR)
        return rc;
    CKN(cudaMemcpyAsync(logits_dev, n->logits,
                        (size_t)B * HL_HEAD_T * HL_HEAD_R * sizeof(float),
                        cudaMemcpyDeviceToDevice, s));
    return HL_NO_ERROR;
}

/* dW and db of layer l from the f32 gradient dy (rows of dy_c values) */
static int layer_dw(hl_net *n, int l, const __nv_bfloat16 *x, const float *dy,
                    int dy_c, int B, cudaStream_t s)
{
    hl_dw_args a;
    memset(&a, 0, sizeof(a));
    a.x = x;
    a.dy = dy;
    a.dy_c = dy_c;
    a.dw = n->g + w_off(l);
    a.db = n->g + b_off(l);
    a.B = B;
    a.H = a.W = l_in_side(l);
    a.Ho = a.Wo = l_out_side(l);
    a.cin = L_CIN[l];
    a.cout = L_COUT[l];
    a.stride = L_STRIDE[l];
    CKN(hl_launch_conv_dw(&a, s));
    return HL_NO_ERROR;
}

/* input gradient of layer l (l >= 1) from the bf16 gradient g of its output */
static int layer_dx(hl_net *n, int l, const __nv_bfloat16 *g, int B,
                    __nv_bfloat16 *dx, cudaStream_t s)
{
    hl_conv_args a;
    memset(&a, 0, sizeof(a));
    a.x = g;
    a.w = n->wb[l];
    a.y = dx;
    a.B = B;
    a.status = n->status;
    if (L_STRIDE[l] == 1) {
        /* dx = conv(g, flipped transposed weights): cin = cout_fwd */
        a.H = a.W = l_out_side(l);
        a.Ho = a.Wo = l_in_side(l);
        a.cin = L_COUT[l];
        a.cout = L_CIN[l];
        a.kreal = 9 * L_COUT[l];
        a.stride = 1;
        CKN(hl_launch_conv3x3(&a, 0, s));
    } else {
        a.H = a.W = l_out_side(l);
        a.Ho = a.Wo = l_in_side(l);
        a.cin = L_COUT[l];
        a.cout = L_CIN[l];
        a.kreal = 9 * L_COUT[l];
        a.stride = 2;
        CKN(hl_launch_conv3x3(&a, 1, s));
    }
    return HL_NO_ERROR;
}

extern "C" int hl_net_train_step(hl_net *n, const void *occ_dev,
                                 const hl_coarse_geom *geo_host,
                                 const float *target_dev, int B, float lr,
                                 float pos_weight, float *loss_host,
                                 void *stream)
{
    if (!n || !occ_dev || !geo_host || !target_dev)
        return HL_NULL_POINTER;
    if (B <= 0)
        return HL_INVALID_DATA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const __nv_bfloat16 *occ = static_cast<const __nv_bfloat16 *>(occ_dev);
    int rc = net_reserve(n, B);
    if (rc != HL_NO_ERROR || (rc = upload_geo(n, geo_host, B, s)) != HL_NO_ERROR)
        return rc;
    if ((rc = net_forward(n, occ, B, s)) != HL_NO_ERROR)
        return rc;
    const int np = n_params();
    CKN(cudaMemsetAsync(n->g, 0, np * sizeof(float), s));
    CKN(cudaMemsetAsync(n->loss, 0, sizeof(float), s));
    const long long cells = (long long)B * HL_HEAD_T * HL_HEAD_R;
    CKN(hl_launch_bce(n->logits, target_dev, n->hsum, cells, pos_weight, n->dz,
                      n->g + ab_off(), n->loss, s));
    CKN(hl_launch_head_bwd(n->dz, NET_EV, n->geo, B, n->w + ab_off(), n->de, s));
    const long long P64 = (long long)B * NET_EV * NET_EV;
    const long long P128 = (long long)B * 128 * 128;
    /* layer 5 (32 -> 1, no ReLU): dW from de, dx = conv(de, flipped W) */
    if ((rc = layer_dw(n, 5, n->act[4], n->de, 1, B, s)) != HL_NO_ERROR)
        return rc;
    CKN(hl_launch_f32_to_bf16(n->de, P64, n->de_b, s));
    {
        hl_conv_args a;
        memset(&a, 0, sizeof(a));
        a.x = n->de_b;
        a.w = n->wb[5];            /* [32][9]: cin 1 -> cout 32, flipped */
        a.y = n->gx;
        a.B = B;
        a.H = a.W = NET_EV;
        a.Ho = a.Wo = NET_EV;
        a.cin = 1;
        a.cout = 32;
        a.kreal = 9;
        a.stride = 1;
        a.status = n->status;
        CKN(hl_launch_conv3x3(&a, 0, s));
    }
    /* layers 4 .. 1 */
    __nv_bfloat16 *gin = n->gx, *gout = n->gx2;
    for (int l = 4; l >= 0; l--) {
        const long long P = (l == 0) ? P128 : P64;
        CKN(hl_launch_relu_mask(gin, n->act[l], P * 32, n->gm, n->gm_b, s));
        const __nv_bfloat16 *xin = (l == 0) ? occ : n->act[l - 1];
        if ((rc = layer_dw(n, l, xin, n->gm, 32, B, s)) != HL_NO_ERROR)
            return rc;
        if (l >= 1) {
            if ((rc = layer_dx(n, l, n->gm_b, B, gout, s)) != HL_NO_ERROR)
                return rc;
            std::swap(gin, gout);
        }
    }
    n->step++;
    if (lr > 0.0f)
        CKN(hl_launch_adam(n->w, n->g, n->m, n->v, np, lr, n->step, 1.0f, s));
    if ((rc = net_refresh(n, s)) != HL_NO_ERROR)
        return rc;
    if (loss_host) {
        float l = 0.0f;
        int st = 0;
        CKN(cudaMemcpyAsync(&l, n->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
        CKN(cudaMemcpyAsync(&st, n->status, sizeof(int), cudaMemcpyDeviceToHost, s));
        CKN(cudaStreamSynchronize(s));
        if (st != 0)
            return HL_CUDA_ERROR;
        *loss_host = l;
    }
    return HL_NO_ERROR;
}

/* Occupancy maps and coarse geometries of device images: each ROI is pooled
 * in f x f cells, f = max(1, ceil(max(w, h) / 256)), into a 256 x 256 bf16
 * map (cells past the ROI are 0); the evidence cell of the network is 4 f
 * pixels and the coarse rho bins split the image's own rho range. */
extern "C" int hl_occupancy(hl_handle *h, const hl_image_desc *imgs, int nimg,
                            void *occ_dev, hl_coarse_geom *geo_host,
                            void *stream)
{
    if (!h || !imgs || !occ_dev || !geo_host)
        return HL_NULL_POINTER;
    if (nimg <= 0)
        return HL_INVALID_DATA;
    std::vector<hl_pool_img> pi((size_t)nimg);
    for (int i = 0; i < nimg; i++) {
        const hl_image_desc &d = imgs[i];
        if (!d.data)
            return HL_NULL_POINTER;
        if (d.roi_x1 < 0 || d.roi_y1 < 0 || d.roi_x2 > d.width || d.roi_y2 > d.height ||
            d.roi_x2 <= d.roi_x1 || d.roi_y2 <= d.roi_y1)
            return HL_INVALID_DATA;
        const int w = d.roi_x2 - d.roi_x1, hh = d.roi_y2 - d.roi_y1;
        const int f = std::max(1, (std::max(w, hh) + NET_IN - 1) / NET_IN);
        pi[i].base = d.data + (size_t)d.roi_y1 * d.pitch + d.roi_x1;
        pi[i].pitch = (long)d.pitch;
        pi[i].w = w;
        pi[i].h = hh;
        pi[i].factor = f;
        pi[i].pad = 0;
        hl_geom g;
        int rc = hl_geometry(h, w, hh, &g);
        if (rc != HL_NO_ERROR)
            return rc;
        hl_coarse_geom &cg = geo_host[i];
        cg.cell = (float)(4 * f);
        cg.rho_min = (float)g.rho_min;
        cg.inv_rw = (float)HL_HEAD_R / (float)g.numrho;
        const int ph = (hh + f - 1) / f, pw = (w + f - 1) / f;
        cg.qh = (ph + 3) / 4;
        cg.qw = (pw + 3) / 4;
        cg.pad = 0;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    hl_pool_img *d_pi = nullptr;
    CKN(cudaMallocAsync(&d_pi, sizeof(hl_pool_img) * nimg, s));
    cudaError_t e = cudaMemcpyAsync(d_pi, pi.data(), sizeof(hl_pool_img) * nimg,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = hl_launch_pool(d_pi, nimg, NET_IN, static_cast<__nv_bfloat16 *>(occ_dev), s);
    cudaFreeAsync(d_pi, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    return cnn_err(e);
}

/* Forward pass for the proposal pipeline: geometry already on the device. */
int hl_net_run(hl_net *n, const __nv_bfloat16 *occ, const hl_head_geom *geo_dev,
               int B, const float **logits, cudaStream_t s)
{
    int rc = net_reserve(n, B);
    if (rc != HL_NO_ERROR)
        return rc;
    CKN(cudaMemcpyAsync(n->geo, geo_dev, (size_t)B * sizeof(hl_head_geom),
                        cudaMemcpyDeviceToDevice, s));
    if ((rc = net_forward(n, occ, B, s)) != HL_NO_ERROR)
        return rc;
    *logits = n->logits;
    return HL_NO_ERROR;
}

int hl_net_status(hl_net *n, int *st, cudaStream_t s)
{
    CKN(cudaMemcpyAsync(st, n->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    return HL_NO_ERROR;
}
