/*
 * ref_runner.c -- runs the REFERENCE's own vote and draw kernels
 * (okano_3_0/HoughLine.cu:86-130 _houghlineImgKer, :133-165
 * _houghlineCorKer, :216-249 _houghoutKer; okano_3_0/HoughCircle.cu:187-245
 * _houghcirImgKer) from the fatbins that oracle/build_ref.sh compiles out of
 * the reference sources, through the CUDA driver API.  TEST INFRASTRUCTURE ONLY: it produces golden accumulators that
 * pin the CPU oracle (tests/golden/make_golden.py).
 *
 * The reference's peak kernels are deliberately never run: their grids are
 * rounded up and they have no bounds check, so they write outside their
 * buffers (_findlocalMaxKer, okano_3_0/HoughLine.cu:791-798, :174-206;
 * _findpartmaxKer, okano_3_0/HoughCircle.cu:321-370, launched at :993).
 *
 * Kernel argument structs restate the layouts of Image / ImageCuda
 * (okano_3_0/Image.h:44-78) and Template (okano_3_0/Template.h:14-20).
 */
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    size_t width, height;
    int roiX1, roiY1, roiX2, roiY2;
    unsigned char *imgData;
} ref_Image;

typedef struct {
    ref_Image imgMeta;
    int deviceId;
    size_t pitchBytes;
} ref_ImageCuda;

typedef struct {
    size_t count;
    int *tplData;
} ref_Template;

typedef struct {
    float angle;
    int distance;
    int votes;
} ref_LineParam;

static CUmodule g_mod, g_cmod;
static CUfunction g_img, g_cor, g_out, g_cvote;
static char g_err[512];

const char *rr_error(void) { return g_err; }

#define DCK(x)                                                           \
    do {                                                                 \
        CUresult r__ = (x);                                              \
        if (r__ != CUDA_SUCCESS) {                                       \
            const char *s__ = NULL;                                      \
            cuGetErrorString(r__, &s__);                                 \
            snprintf(g_err, sizeof(g_err), "%s: %s (line %d)", #x,       \
                     s__ ? s__ : "?", __LINE__);                         \
            return -7;                                                   \
        }                                                                \
    } while (0)

/* Find a kernel by a fragment of its name among the module's functions. */
static int find_fn(CUmodule mod, const char *frag, CUfunction *out)
{
    unsigned n = 0;
    DCK(cuModuleGetFunctionCount(&n, mod));
    CUfunction *fs = (CUfunction *)calloc(n ? n : 1, sizeof(CUfunction));
    if (!fs)
        return -6;
    CUresult r = cuModuleEnumerateFunctions(fs, n, mod);
    if (r != CUDA_SUCCESS) {
        free(fs);
        snprintf(g_err, sizeof(g_err), "cuModuleEnumerateFunctions failed");
        return -7;
    }
    int found = -1;
    for (unsigned i = 0; i < n; i++) {
        const char *nm = NULL;
        if (cuFuncGetName(&nm, fs[i]) == CUDA_SUCCESS && nm &&
            strstr(nm, frag)) {
            *out = fs[i];
            found = 0;
            break;
        }
    }
    free(fs);
    if (found)
        snprintf(g_err, sizeof(g_err), "kernel %s not found", frag);
    return found;
}

/* Load the fatbin into the primary context of device 0 (shared with the
 * CUDA runtime of the calling process). */
int rr_init(const char *fatbin_path)
{
    if (g_mod)
        return 0;
    CUdevice dev;
    CUcontext ctx;
    DCK(cuInit(0));
    DCK(cuDeviceGet(&dev, 0));
    DCK(cuDevicePrimaryCtxRetain(&ctx, dev));
    DCK(cuCtxSetCurrent(ctx));
    DCK(cuModuleLoad(&g_mod, fatbin_path));
    if (find_fn(g_mod, "_houghlineImgKer", &g_img))
        return -7;
    if (find_fn(g_mod, "_houghlineCorKer", &g_cor))
        return -7;
    if (find_fn(g_mod, "_houghoutKer", &g_out))
        return -7;
    return 0;
}

/* Load the HoughCircle fatbin into the same context (after rr_init). */
int rr_init_circle(const char *fatbin_path)
{
    if (g_cmod)
        return 0;
    if (!g_mod) {
        snprintf(g_err, sizeof(g_err), "rr_init has not run");
        return -7;
    }
    DCK(cuModuleLoad(&g_cmod, fatbin_path));
    if (find_fn(g_cmod, "_houghcirImgKer", &g_cvote))
        return -7;
    return 0;
}

/* Vote an ROI of a host image with the reference's _houghcirImgKer, launched
 * as okano_3_0/HoughCircle.cu:964-977 does (32 x 8 blocks over the ROI, one
 * grid layer per radius, the ROI sub-image of :956).  acc receives the
 * reference's zero-bordered buffer, (rmax - rmin + 1) planes of
 * (roi_h + 2) x (roi_w + 2) ints. */
int rr_circle_vote(const uint8_t *img, int width, int height, long pitch,
                   int x1, int y1, int x2, int y2, int rmin, int rmax, int32_t *acc)
{
    int bw = x2 - x1, bh = y2 - y1;
    const int nr = rmax - rmin + 1;
    if (!g_cvote || bw <= 0 || bh <= 0 || rmin < 0 || nr <= 0 || nr > 65535) {
        snprintf(g_err, sizeof(g_err), "bad circle vote arguments");
        return -1;
    }
    size_t dpitch = ((size_t)width + 511) / 512 * 512;
    size_t accn = (size_t)nr * (size_t)(bw + 2) * (size_t)(bh + 2);
    CUdeviceptr dimg = 0, dacc = 0;
    DCK(cuMemAlloc(&dimg, dpitch * (size_t)height));
    DCK(cuMemAlloc(&dacc, accn * 4));
    DCK(cuMemsetD32(dacc, 0, accn));
    CUDA_MEMCPY2D cp;
    memset(&cp, 0, sizeof(cp));
    cp.srcMemoryType = CU_MEMORYTYPE_HOST;
    cp.srcHost = img;
    cp.srcPitch = (size_t)pitch;
    cp.dstMemoryType = CU_MEMORYTYPE_DEVICE;
    cp.dstDevice = dimg;
    cp.dstPitch = dpitch;
    cp.WidthInBytes = (size_t)width;
    cp.Height = (size_t)height;
    DCK(cuMemcpy2D(&cp));
    ref_ImageCuda sub;
    memset(&sub, 0, sizeof(sub));
    sub.imgMeta.width = (size_t)bw;
    sub.imgMeta.height = (size_t)bh;
    sub.imgMeta.roiX1 = x1;
    sub.imgMeta.roiY1 = y1;
    sub.imgMeta.roiX2 = x2;
    sub.imgMeta.roiY2 = y2;
    sub.imgMeta.imgData = (unsigned char *)(uintptr_t)(dimg + (size_t)y1 * dpitch + (size_t)x1);
    sub.pitchBytes = dpitch;
    int radius_min = rmin;
    void *args[] = {&sub, &dacc, &radius_min, &bw, &bh};
    DCK(cuLaunchKernel(g_cvote, (unsigned)((bw + 31) / 32), (unsigned)((bh + 7) / 8),
                       (unsigned)nr, 32, 8, 1, 0, 0, args, NULL));
    DCK(cuCtxSynchronize());
    DCK(cuMemcpyDtoH(acc, dacc, accn * 4));
    cuMemFree(dimg);
    cuMemFree(dacc);
    return 0;
}

static int ref_dims(int w, int h, double detheta, double derho, int *T, int *R)
{
    /* okano_3_0/HoughLine.cu:670-671 */
    *R = (int)((double)(int)((w + h) * 2 + 1) / derho);
    *T = (int)(3.14159265358979323846 / detheta);
    return 0;
}

/* Vote an ROI of a host image with the reference kernel.  acc receives the
 * reference's padded accumulator (T + 2) x (numrho + 2) ints. */
int rr_vote_image(const uint8_t *img, int width, int height, long pitch,
                  int x1, int y1, int x2, int y2, double detheta,
                  double derho, int32_t *acc)
{
    int T, R;
    ref_dims(x2 - x1, y2 - y1, detheta, derho, &T, &R);
    size_t dpitch = ((size_t)width + 511) / 512 * 512;
    CUdeviceptr dimg = 0, dacc = 0;
    size_t accn = (size_t)(T + 2) * (size_t)(R + 2);
    DCK(cuMemAlloc(&dimg, dpitch * (size_t)height));
    DCK(cuMemAlloc(&dacc, accn * 4));
    DCK(cuMemsetD32(dacc, 0, accn));
    CUDA_MEMCPY2D cp;
    memset(&cp, 0, sizeof(cp));
    cp.srcMemoryType = CU_MEMORYTYPE_HOST;
    cp.srcHost = img;
    cp.srcPitch = (size_t)pitch;
    cp.dstMemoryType = CU_MEMORYTYPE_DEVICE;
    cp.dstDevice = dimg;
    cp.dstPitch = dpitch;
    cp.WidthInBytes = (size_t)width;
    cp.Height = (size_t)height;
    DCK(cuMemcpy2D(&cp));
    /* roiSubImage, okano_3_0/Image.h:218-258 */
    ref_ImageCuda sub;
    memset(&sub, 0, sizeof(sub));
    sub.imgMeta.width = (size_t)(x2 - x1);
    sub.imgMeta.height = (size_t)(y2 - y1);
    sub.imgMeta.roiX1 = x1;
    sub.imgMeta.roiY1 = y1;
    sub.imgMeta.roiX2 = x2;
    sub.imgMeta.roiY2 = y2;
    sub.imgMeta.imgData = (unsigned char *)(uintptr_t)(dimg + (size_t)y1 * dpitch + (size_t)x1);
    sub.deviceId = 0;
    sub.pitchBytes = dpitch;
    CUdeviceptr bufhough = dacc + 4;   /* alldatadev + 1 holds sum, :690-692 */
    (void)bufhough;
    CUdeviceptr hough = dacc;
    int numtheta = T, numrho = R;
    void *args[] = {&sub, &hough, &numtheta, &numrho, &detheta, &derho};
    unsigned gx = (unsigned)((x2 - x1 + 31) / 32), gy = (unsigned)((y2 - y1 + 7) / 8);
    DCK(cuLaunchKernel(g_img, gx, gy, 1, 32, 8, 1, 0, 0, args, NULL));
    DCK(cuCtxSynchronize());
    DCK(cuMemcpyDtoH(acc, dacc, accn * 4));
    cuMemFree(dimg);
    cuMemFree(dacc);
    return 0;
}

/* Vote an interleaved (x, y) list with the reference kernel.  n must be a
 * multiple of 16: the reference grid is rounded up to 16 threads and has no
 * bounds check on the index (okano_3_0/HoughLine.cu:138-142, :720-723).
 * w, h: the extents the reference derives from the bounding box. */
int rr_vote_points(const int *xy, int n, int w, int h, double detheta,
                   double derho, int32_t *acc)
{
    if (n <= 0 || (n % 16) != 0) {
        snprintf(g_err, sizeof(g_err), "n must be a positive multiple of 16");
        return -1;
    }
    int T, R;
    ref_dims(w, h, detheta, derho, &T, &R);
    size_t accn = (size_t)(T + 2) * (size_t)(R + 2);
    CUdeviceptr dxy = 0, dacc = 0;
    DCK(cuMemAlloc(&dxy, sizeof(int) * 2 * (size_t)n));
    DCK(cuMemAlloc(&dacc, accn * 4));
    DCK(cuMemsetD32(dacc, 0, accn));
    DCK(cuMemcpyHtoD(dxy, xy, sizeof(int) * 2 * (size_t)n));
    ref_Template t;
    t.count = (size_t)n;
    t.tplData = (int *)(uintptr_t)dxy;
    int numtheta = T, numrho = R;
    void *args[] = {&t, &dacc, &numtheta, &numrho, &detheta, &derho};
    DCK(cuLaunchKernel(g_cor, (unsigned)(n / 16), 1, 1, 16, 1, 1, 0, 0, args,
                       NULL));
    DCK(cuCtxSynchronize());
    DCK(cuMemcpyDtoH(acc, dacc, accn * 4));
    cuMemFree(dxy);
    cuMemFree(dacc);
    return 0;
}

/* Draw lines with the reference kernel on a zeroed w x h image; out is
 * w x h bytes (host, pitch w). */
int rr_draw_lines(const float *angle, const int *distance, int nlines,
                  int w, int h, int derho, uint8_t *out)
{
    size_t dpitch = ((size_t)w + 511) / 512 * 512;
    CUdeviceptr dimg = 0, dl = 0;
    DCK(cuMemAlloc(&dimg, dpitch * (size_t)h));
    DCK(cuMemsetD8(dimg, 0, dpitch * (size_t)h));
    ref_LineParam *lp = (ref_LineParam *)calloc((size_t)(nlines > 0 ? nlines : 1),
                                                sizeof(ref_LineParam));
    if (!lp)
        return -6;
    for (int i = 0; i < nlines; i++) {
        lp[i].angle = angle[i];
        lp[i].distance = distance[i];
        lp[i].votes = 1;
    }
    DCK(cuMemAlloc(&dl, sizeof(ref_LineParam) * (size_t)(nlines > 0 ? nlines : 1)));
    DCK(cuMemcpyHtoD(dl, lp, sizeof(ref_LineParam) * (size_t)(nlines > 0 ? nlines : 1)));
    free(lp);
    ref_ImageCuda o;
    memset(&o, 0, sizeof(o));
    o.imgMeta.width = (size_t)w;
    o.imgMeta.height = (size_t)h;
    o.imgMeta.roiX2 = w;
    o.imgMeta.roiY2 = h;
    o.imgMeta.imgData = (unsigned char *)(uintptr_t)dimg;
    o.pitchBytes = dpitch;
    void *args[] = {&o, &dl, &nlines, &derho};
    DCK(cuLaunchKernel(g_out, (unsigned)((w + 31) / 32), (unsigned)((h + 7) / 8), 1,
                       32, 8, 1, 0, 0, args, NULL));
    DCK(cuCtxSynchronize());
    CUDA_MEMCPY2D cp;
    memset(&cp, 0, sizeof(cp));
    cp.srcMemoryType = CU_MEMORYTYPE_DEVICE;
    cp.srcDevice = dimg;
    cp.srcPitch = dpitch;
    cp.dstMemoryType = CU_MEMORYTYPE_HOST;
    cp.dstHost = out;
    cp.dstPitch = (size_t)w;
    cp.WidthInBytes = (size_t)w;
    cp.Height = (size_t)h;
    DCK(cuMemcpy2D(&cp));
    cuMemFree(dimg);
    cuMemFree(dl);
    return 0;
}
