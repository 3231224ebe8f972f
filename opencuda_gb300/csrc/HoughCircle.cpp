/*
 * HoughCircle.cpp -- the drop-in HoughCircle class (include/HoughCircle.h)
 * over the C ABI.  Each method keeps the reference's argument checks, its
 * in-place migration of the input image / point set to the current device,
 * and its ErrorCode returns, then hands the work to hl_circles.
 */
#include <string.h>

#include <vector>

#include <cuda_runtime.h>

#include "HoughCircle.h"
#include "hl_circle.h"
#include "houghline_gb300.h"

static_assert(sizeof(CircleParam) == sizeof(hl_circle), "CircleParam layout");

HoughCircle &HoughCircle::operator=(const HoughCircle &o)
{
    if (this != &o) {
        radiusMin = o.radiusMin;
        radiusMax = o.radiusMax;
        distThres = o.distThres;
        rThres = o.rThres;
        cirThreshold = o.cirThreshold;
    }
    return *this;
}

HoughCircle::~HoughCircle()
{
    if (gpu_)
        hl_destroy(gpu_);
}

/* the workspace (its line parameters are unused by the circle path) */
int HoughCircle::ensure() const
{
    if (gpu_)
        return NO_ERROR;
    hl_params p;
    p.detheta = 3.14159265358979323846 / 180;
    p.derho = 1.0;
    p.threshold = 90;
    p.thresang = (float)(3.14159265358979323846 / 180 * 5.0f);
    p.thresdis = 50;
    return hl_create(&gpu_, &p);
}

static void desc_of(Image *img, hl_image_desc *d)
{
    ImageCuda *c = IMAGE_CUDA(img);
    d->data = img->imgData;
    d->pitch = c->pitchBytes;
    d->width = (int)img->width;
    d->height = (int)img->height;
    d->roi_x1 = img->roiX1;
    d->roi_y1 = img->roiY1;
    d->roi_x2 = img->roiX2;
    d->roi_y2 = img->roiY2;
}

int HoughCircle::houghcircle(Image *inimg, CoordiSet *guidingset, int *circleMax,
                             CircleParam *circleparam, bool writetofile)
{
    (void)writetofile;
    if (inimg == NULL && guidingset == NULL)                /* :1241-1242 */
        return NULL_POINTER;
    if (!circleMax)
        return NULL_POINTER;
    int rc = ensure();
    if (rc != NO_ERROR)
        return rc;
    hl_circle_params p;
    p.radius_min = radiusMin;
    p.radius_max = radiusMax;
    p.dist_thres = distThres;
    p.r_thres = (int)rThres;
    p.threshold = cirThreshold;
    hl_circle *out = reinterpret_cast<hl_circle *>(circleparam);
    if (guidingset == NULL) {
        rc = ImageBasicOp::copyToCurrentDevice(inimg);      /* :944 */
        if (rc != NO_ERROR)
            return rc;
        hl_image_desc d;
        desc_of(inimg, &d);
        return hl_circles(gpu_, &d, &p, circleMax, out, NULL);
    }
    /* :1251-1281: the set migrates to the device; its points are drawn as
     * 255 into a zero image of (max x + 2) x (max y + 2) */
    if (guidingset->count == 0)
        return INVALID_DATA;
    rc = CoordiSetBasicOp::copyToCurrentDevice(guidingset);
    if (rc != NO_ERROR)
        return rc;
    const size_t n = guidingset->count;
    std::vector<int> xy(2 * n);
    if (cudaMemcpy(xy.data(), guidingset->tplData, sizeof(int) * 2 * n,
                   cudaMemcpyDeviceToHost) != cudaSuccess)
        return CUDA_ERROR;
    int maxx = xy[0], maxy = xy[1];
    for (size_t i = 1; i < n; i++) {
        maxx = xy[2 * i] > maxx ? xy[2 * i] : maxx;
        maxy = xy[2 * i + 1] > maxy ? xy[2 * i + 1] : maxy;
    }
    if (maxx < 0 || maxy < 0 || maxx + 2 > HL_MAX_SIDE || maxy + 2 > HL_MAX_SIDE)
        return INVALID_DATA;
    Image *coor = NULL;
    ImageBasicOp::newImage(&coor);
    rc = ImageBasicOp::makeAtHost(coor, maxx + 2, maxy + 2);
    if (rc == NO_ERROR) {
        memset(coor->imgData, 0, (size_t)(maxx + 2) * (size_t)(maxy + 2));
        for (size_t i = 0; i < n; i++) {
            const int x = xy[2 * i], y = xy[2 * i + 1];
            if (x >= 0 && y >= 0)
                coor->imgData[(size_t)y * (size_t)(maxx + 2) + (size_t)x] = 255;
        }
        rc = ImageBasicOp::copyToCurrentDevice(coor);
    }
    if (rc == NO_ERROR) {
        hl_image_desc d;
        desc_of(coor, &d);
        rc = hl_circles(gpu_, &d, &p, circleMax, out, NULL);
    }
    ImageBasicOp::deleteImage(coor);
    return rc;
}

int HoughCircle::pieceCircle(Image *inimg, int piecenum, int *circleMax,
                             CircleParam *circleparam, bool writetofile)
{
    (void)writetofile;
    if (!inimg || !circleMax)
        return NULL_POINTER;
    if (piecenum <= 0 || piecenum > 4096)
        return INVALID_DATA;
    int rc = ensure();
    if (rc != NO_ERROR)
        return rc;
    rc = ImageBasicOp::copyToCurrentDevice(inimg);
    if (rc != NO_ERROR)
        return rc;
    /* the pieces of :1340-1352 (ROI [x * c, x * c + c - 1), 10 circles
     * each), all in one hl_circles_batch call */
    const int cx = (int)inimg->width / piecenum, cy = (int)inimg->height / piecenum;
    const int np = piecenum * piecenum;
    std::vector<hl_image_desc> d((size_t)np);
    for (int y = 0; y < piecenum; y++)
        for (int x = 0; x < piecenum; x++) {
            inimg->roiX1 = x * cx;
            inimg->roiX2 = x * cx + cx - 1;
            inimg->roiY1 = y * cy;
            inimg->roiY2 = y * cy + cy - 1;
            desc_of(inimg, &d[(size_t)y * piecenum + x]);
        }
    hl_circle_params p;
    p.radius_min = radiusMin;
    p.radius_max = radiusMax;
    p.dist_thres = distThres;
    p.r_thres = (int)rThres;
    p.threshold = cirThreshold;
    std::vector<hl_circle> res((size_t)np * 10);
    std::vector<int> cnt((size_t)np);
    rc = hl_circles_batch(gpu_, d.data(), np, &p, 10, res.data(), cnt.data(), NULL);
    /* the reference ignores each piece's return code and keeps the other
     * pieces' circles (:1366-1375); a piece with more local maxima than the
     * candidate buffer holds (OP_OVERFLOW) contributes none here, its count
     * being 0, and the rest are kept */
    if (rc != NO_ERROR && rc != OP_OVERFLOW)
        return rc;
    int pointer = 0;
    for (int i = 0; i < np; i++)
        for (int k = 0; k < cnt[i] && pointer < *circleMax; k++)
            circleparam[pointer++] = *reinterpret_cast<const CircleParam *>(&res[(size_t)i * 10 + k]);
    *circleMax = pointer;
    return NO_ERROR;
}
