/*
 * hl_window.h -- argument blocks of the proposal-guided vote (not part of
 * the C ABI).
 */
#ifndef HL_WINDOW_H
#define HL_WINDOW_H

#include "hl_internal.h"

/* coarse grid of the proposal head */
#define HL_COARSE_T 90
#define HL_COARSE_R 128
/* tiles one window may filter (64 Mpixel ROIs) */
#define HL_WIN_MAXTILES 16384
/* thetas of a window whose cos / sin the vote keeps in shared memory */
#define HL_WIN_MAXK 64
/* hit tiles of a window listed for the warps (more: taken by mask word) */
#define HL_WIN_HITS 4096
/* rho cells one window may span (a run of marked cells at one theta) */
#define HL_WIN_RUN 8

typedef struct hl_select_args {
    const float *logits;   /* [nimg][90][128] */
    float zcut;            /* logit of the probability cutoff */
    int max_props;         /* more candidates above the cutoff: fall back */
    int top_m;             /* also take each image's top_m candidates (0: none) */
    int dil_t, dil_r;      /* window dilation in coarse cells */
    int force_fallback;
    int nms;               /* candidates: local maxima of the logits (else every cell) */
    int use_conf;          /* confidence test on (zconf) */
    float zconf;           /* fall back when the best unselected candidate is above */
    int *fallback;         /* out [nimg]: 0, 1 (count test) or 2 (confidence test) */
    int4 *win;             /* out: {image, t, r, r1}: rho cells r .. r1 */
    int *nwin;             /* window counter (zeroed before) */
    int *ncells;           /* marked coarse cells (zeroed before) */
    int cap;
    int *status;
} hl_select_args;

typedef struct hl_window_args {
    const int4 *win;
    const int *nwin;
    int cap;
    const hl_vote_img *vimgs;
    const hl_peak_img *pimgs;
    const float *cosv, *sinv;
    int T;
    float irho;
    unsigned long long *votes;   /* executed votes, or NULL */
    int *status;
    /* 6 or 10: every window has at most that many thetas and the vote may
     * take the branch-free path compiled for it (its accumulator has room
     * for that many columns); 0: the general path */
    int nk_fast;
} hl_window_args;

cudaError_t hl_launch_select(const hl_select_args *a, int nimg, cudaStream_t s);
cudaError_t hl_launch_window_vote(const hl_window_args *a, int max_win_bins,
                                  int grid, cudaStream_t s);

#endif
