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

/* ---- the network --------------------------------------------------------
 * Input: a 256 x 256 occupancy map per image (bf16, the fraction of edge
 * pixels in each f x f cell, hl_occupancy).  Six 3x3 convolutions with
 * padding 1: 1 -> 32 (stride 2), 32 -> 32 (stride 2), three 32 -> 32, then
 * 32 -> 1, ReLU after all but the last: a 64 x 64 evidence map.  The fixed
 * coarse Hough head sums the evidence of every cell into 90 angle x 128 rho
 * bins of the image's own rho range; logits = alpha * sums + beta.  FP32
 * master weights (flat: per layer W [cout][9 * cin] then b [cout], then
 * alpha, beta), BF16 copies for the tensor cores. */
typedef struct hl_net hl_net;

/* Coarse geometry of one image: evidence cell size in pixels, rho range
 * start, coarse bins per rho unit, evidence cells covering the ROI. */
typedef struct hl_coarse_geom {
    float cell;
    float rho_min;
    float inv_rw;
    int qh, qw;
    int pad;
} hl_coarse_geom;

int hl_net_create(hl_net **out, unsigned long long seed);
int hl_net_destroy(hl_net *net);
int hl_net_num_params(void);
int hl_net_get_params(hl_net *net, float *host);
int hl_net_set_params(hl_net *net, const float *host);
/* gradients of the last hl_net_train_step (host copy, num_params floats) */
int hl_net_get_grads(hl_net *net, float *host);

/* occ_dev [B][256][256] bf16 -> logits_dev [B][90][128] f32 */
int hl_net_forward(hl_net *net, const void *occ_dev,
                   const hl_coarse_geom *geo_host, int B, float *logits_dev,
                   void *stream);

/* One step on a batch: forward, weighted binary cross-entropy against
 * target_dev [B][90][128] (1 where a line of the plain method lies, else 0;
 * positives weighted by pos_weight, mean over cells), backward with the
 * project's kernels (tensor-core input gradients, FP32 weight gradients),
 * Adam (lr; gradients clipped to +-1; lr = 0 leaves the weights).  Writes
 * the loss to *loss_host when not NULL (then synchronises). */
int hl_net_train_step(hl_net *net, const void *occ_dev,
                      const hl_coarse_geom *geo_host, const float *target_dev,
                      int B, float lr, float pos_weight, float *loss_host,
                      void *stream);

/* Occupancy maps [nimg][256][256] bf16 and coarse geometries of DEVICE
 * images (the handle gives the rho layout).  Synchronises. */
int hl_occupancy(hl_handle *h, const hl_image_desc *imgs, int nimg,
                 void *occ_dev, hl_coarse_geom *geo_host, void *stream);

/* ---- proposal-guided batched HoughLine ------------------------------------
 * hl_batch's contract (DEVICE images, per-image thresholds, linesmax lines
 * per image into DEVICE arrays), but the exact vote runs only in the coarse
 * cells the network selects: the candidates (every cell, or with nms the
 * local maxima of the logits over 3 x 3 cells) scored above p_cut, and with
 * top_m > 0 also the image's top_m candidates whatever their score, each
 * grown by dilate_theta / dilate_rho cells.  Every reported line is a peak of
 * the full accumulator with its exact vote count; lines the proposals miss
 * are absent.  An image runs the full plain method instead when the network
 * is not confident its budget covers the lines: more than max_props
 * candidates above p_cut (a cluttered scene), or, with 0 < p_conf < 1, the
 * best candidate left out of the top_m scored above p_conf; an image too
 * large for the window kernel falls back too.  Every judge_every-th other
 * image (0: none) also runs the plain method and the stats report how many
 * of its lines the proposal path found.  Synchronises `stream` (the
 * fall-back set is decided on the host). */
typedef struct hl_proposal_opts {
    float p_cut;
    int max_props;
    int dilate_theta;
    int dilate_rho;
    int judge_every;
    int top_m;          /* also vote each image's top_m candidates (0: none) */
    int nms;            /* candidates are the local maxima of the logits */
    float p_conf;       /* confidence fall-back threshold (0: off) */
} hl_proposal_opts;

typedef struct hl_proposal_stats {
    int fallback;        /* images that ran the plain method instead */
    int windows;         /* windows voted (runs of up to 8 coarse cells) */
    int judged;          /* images also run through the plain method */
    int judged_lines;    /* lines the plain method gave them */
    int judged_found;    /* of those, reported by the proposal path */
    int fallback_conf;   /* of the fall-backs, decided by the confidence test */
    long long votes;     /* executed votes of the windows */
    int cells;           /* coarse cells the windows cover */
    int pad;
} hl_proposal_stats;

int hl_proposal_batch(hl_handle *h, hl_net *net, const hl_image_desc *imgs,
                      int nimg, const int *thresholds, int linesmax,
                      const hl_proposal_opts *opts, hl_line *lines_dev,
                      int *counts_dev, hl_proposal_stats *stats, void *stream);

/* The seeded scene generator (hl_synth_scene) run on the GPU, one CTA per
 * scene, for training data: outs[i].data (DEVICE, pitch outs[i].pitch, at
 * least params[i].width x height) receives exactly the bytes
 * hl_synth_scene(&params[i], ...) writes on the host.  Synchronises. */
int hl_synth_scenes_device(const hl_scene_params *params, int n,
                           const hl_image_desc *outs, void *stream);

#ifdef __cplusplus
}
#endif
#endif
