/*
 * hl_noalloc.cu -- edge-pixel compaction (stage (a)) for callers that must
 * not allocate device memory.
 *
 * Some callers cannot call cudaMalloc once they are running: applications
 * that hand the whole device to their own memory manager or work inside a
 * fixed device-memory budget set at start-up, and latency-bound loops that
 * cannot afford an allocation (cudaMalloc may wait for work already queued
 * on the device).  They still own the inputs and outputs.  The compaction
 * kernel needs scratch for its decoupled look-back (one state word per
 * 128 x 32 tile, a tile ticket, a status word); hl_compact keeps that scratch
 * in a handle, which allocates.  hl_compact_noalloc instead keeps it in the
 * file-scope device array below, which every GPU that loads this library
 * holds until the process exits, and launches the same compaction kernel on
 * it.  The kernel keeps one look-back state per group of HL_COMPACT_GROUP
 * tiles, so the array holds HL_NOALLOC_MAX_TILES / HL_COMPACT_GROUP states
 * plus two counters (about 128 KiB).  hl_compact_noalloc_status reads the
 * status word the last call left in it.
 */
#include <mutex>

#include <string.h>

#include "hl_internal.h"

#define NOALLOC_MAX_GROUPS (HL_NOALLOC_MAX_TILES / HL_COMPACT_GROUP)

/* [0] group ticket, [1] status word, [2 ..] one look-back state per group
 * of HL_COMPACT_GROUP tiles */
static __device__ __align__(256) unsigned long long
    g_noalloc_scratch[NOALLOC_MAX_GROUPS + 2];

/* Host-side stand-in of the array above: its name is not a device address in
 * host code, so each device's address is looked up once, with that device
 * current, and cached here. */
#define NOALLOC_MAX_DEVICES 64
static unsigned long long *g_scratch_ptr[NOALLOC_MAX_DEVICES];
static std::mutex g_scratch_mu;

static int scratch_for_current_device(unsigned long long **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return HL_CUDA_ERROR;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return HL_OP_OVERFLOW;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
            return HL_CUDA_ERROR;
        g_scratch_ptr[dev] = static_cast<unsigned long long *>(p);
    }
    *out = g_scratch_ptr[dev];
    return HL_NO_ERROR;
}

extern "C" int hl_compact_noalloc(const hl_image_desc *img, uint32_t *pts_dev,
                                  int *tile_off_dev, int *count_dev,
                                  void *stream)
{
    if (!img || !img->data || !pts_dev || !tile_off_dev || !count_dev)
        return HL_NULL_POINTER;
    if (img->width <= 0 || img->height <= 0 || img->pitch < (size_t)img->width ||
        img->roi_x1 < 0 || img->roi_y1 < 0 || img->roi_x2 > img->width ||
        img->roi_y2 > img->height || img->roi_x2 <= img->roi_x1 ||
        img->roi_y2 <= img->roi_y1)
        return HL_INVALID_DATA;
    const int w = img->roi_x2 - img->roi_x1, h = img->roi_y2 - img->roi_y1;
    if (w > HL_MAX_SIDE || h > HL_MAX_SIDE)
        return HL_INVALID_DATA;
    const int tiles_x = (w + HL_TILE_W - 1) / HL_TILE_W;
    const long long ntiles = (long long)tiles_x * ((h + HL_TILE_H - 1) / HL_TILE_H);
    const long long ngroups = (ntiles + HL_COMPACT_GROUP - 1) / HL_COMPACT_GROUP;
    if (ngroups > NOALLOC_MAX_GROUPS)
        return HL_OP_OVERFLOW;   /* the ROI needs more look-back states */
    unsigned long long *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != HL_NO_ERROR)
        return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    /* the array keeps the previous call's contents: the ticket, the status
     * and the group states this call uses start from zero */
    if (cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * (size_t)(ngroups + 2),
                        s) != cudaSuccess)
        return HL_CUDA_ERROR;
    hl_compact_args ca;
    memset(&ca, 0, sizeof(ca));
    ca.roi.base = img->data + (size_t)img->roi_y1 * img->pitch + img->roi_x1;
    ca.roi.pitch = (long)img->pitch;
    ca.roi.w = w;
    ca.roi.h = h;
    ca.tiles_x = tiles_x;
    ca.ntiles = (int)ntiles;
    ca.imgs = nullptr;
    ca.group_img = nullptr;
    ca.nimg = 0;
    ca.ngroups = 0;
    ca.ticket = reinterpret_cast<unsigned *>(scratch);
    ca.ticket_base = 0;
    ca.status = reinterpret_cast<int *>(scratch + 1);
    ca.tile_state = scratch + 2;
    ca.epoch = 1;
    ca.pts = pts_dev;
    ca.pts_f2 = nullptr;
    ca.tile_off = tile_off_dev;
    ca.count = count_dev;
    return hl_launch_compact(&ca, s) == cudaSuccess ? HL_NO_ERROR : HL_CUDA_ERROR;
}

extern "C" int hl_compact_noalloc_status(int *status, void *stream)
{
    if (!status)
        return HL_NULL_POINTER;
    unsigned long long *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != HL_NO_ERROR)
        return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int v = 0;
    if (cudaMemcpyAsync(&v, scratch + 1, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return HL_CUDA_ERROR;
    *status = v;
    return HL_NO_ERROR;
}
