/*
 * HoughLine.cpp -- the drop-in HoughLine class (include/HoughLine.h) over the
 * C ABI.  Each method keeps the reference's argument checks, its in-place
 * migration of the input image / point set to the current device, and its
 * ErrorCode returns, then hands the work to libhoughline_gb300's kernels.
 */
#include <math.h>
#include <string.h>

#include "HoughLine.h"
#include "houghline_gb300.h"

static_assert(sizeof(LineParam) == sizeof(hl_line), "LineParam layout");

HoughLine &HoughLine::operator=(const HoughLine &o)
{
    if (this != &o) {
        detheta = o.detheta;
        derho = o.derho;
        threshold = o.threshold;
        thresang = o.thresang;
        thresdis = o.thresdis;
    }
    return *this;
}

HoughLine::~HoughLine()
{
    if (gpu_)
        hl_destroy(gpu_);
}

/* create the workspace on first use; push setter changes to it */
int HoughLine::sync_params() const
{
    hl_params p;
    p.detheta = detheta;
    p.derho = derho;
    p.threshold = threshold;
    p.thresang = thresang;
    p.thresdis = thresdis;
    if (!gpu_)
        return hl_create(&gpu_, &p);
    hl_params cur;
    hl_get_params(gpu_, &cur);
    if (cur.detheta != p.detheta || cur.derho != p.derho ||
        cur.threshold != p.threshold || cur.thresang != p.thresang ||
        cur.thresdis != p.thresdis)
        return hl_set_params(gpu_, &p);
    return NO_ERROR;
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

int HoughLine::houghLineCor(CoordiSet *guidingset, int *linesmax,
                            LineParam *lineparam)
{
    if (!guidingset || !linesmax)
        return NULL_POINTER;
    if (guidingset->count == 0 || guidingset->count > 0x7fffffff)
        return INVALID_DATA;
    int rc = sync_params();
    if (rc != NO_ERROR)
        return rc;
    rc = CoordiSetBasicOp::copyToCurrentDevice(guidingset);   /* :422 */
    if (rc != NO_ERROR)
        return rc;
    return hl_plain_points(gpu_, guidingset->tplData, (int)guidingset->count,
                           linesmax, reinterpret_cast<hl_line *>(lineparam), NULL);
}

int HoughLine::houghLine(Image *inimg, CoordiSet *guidingset, int *linesmax,
                         LineParam *lineparam)
{
    if (inimg == NULL && guidingset == NULL)            /* :640-641 */
        return NULL_POINTER;
    if (guidingset != NULL)                              /* set wins, :651 */
        return houghLineCor(guidingset, linesmax, lineparam);
    if (!linesmax)
        return NULL_POINTER;
    int rc = sync_params();
    if (rc != NO_ERROR)
        return rc;
    rc = ImageBasicOp::copyToCurrentDevice(inimg);      /* :736 */
    if (rc != NO_ERROR)
        return rc;
    hl_image_desc d;
    desc_of(inimg, &d);
    return hl_plain(gpu_, &d, linesmax, reinterpret_cast<hl_line *>(lineparam),
                    NULL);
}

int HoughLine::houghLineImg(Image *inimg, CoordiSet *guidingset, Image *outimg,
                            int *linesmax, LineParam *lineparam)
{
    if (inimg == NULL && guidingset == NULL)
        return NULL_POINTER;
    if (!linesmax || !outimg)
        return NULL_POINTER;
    int rc = sync_params();
    if (rc != NO_ERROR)
        return rc;
    if (guidingset != NULL) {
        /* the reference draws through an output view it never set up on
         * this branch; here the lines go to the output image's ROI */
        rc = houghLineCor(guidingset, linesmax, lineparam);
        if (rc != NO_ERROR)
            return rc;
        if ((rc = ImageBasicOp::copyToCurrentDevice(outimg)) != NO_ERROR)
            return rc;
        hl_image_desc dout;
        desc_of(outimg, &dout);
        return hl_draw_lines(gpu_, &dout,
                             reinterpret_cast<const hl_line *>(lineparam),
                             *linesmax, NULL);
    }
    if ((rc = ImageBasicOp::copyToCurrentDevice(inimg)) != NO_ERROR)   /* :1071 */
        return rc;
    if (ImageBasicOp::copyToCurrentDevice(outimg) != NO_ERROR) {       /* :1076-1085 */
        rc = ImageBasicOp::makeAtCurrentDevice(outimg, inimg->roiX2 - inimg->roiX1,
                                               inimg->roiY2 - inimg->roiY1);
        if (rc != NO_ERROR)
            return rc;
    }
    hl_image_desc din, dout;
    desc_of(inimg, &din);
    desc_of(outimg, &dout);
    return hl_plain_draw(gpu_, &din, &dout, linesmax,
                         reinterpret_cast<hl_line *>(lineparam), NULL);
}

bool HoughLine::realLine(Image *inimg, int x1, int y1, int x2, int y2,
                         float threshold, float thresperc)
{
    if (!inimg || sync_params() != NO_ERROR)
        return false;
    if (ImageBasicOp::copyToCurrentDevice(inimg) != NO_ERROR)   /* :1419 */
        return false;
    hl_image_desc d;
    desc_of(inimg, &d);
    int real = 0;
    if (hl_real_line(gpu_, &d, x1, y1, x2, y2, threshold, thresperc, &real, NULL,
                     NULL) != HL_NO_ERROR)
        return false;
    return real != 0;
}

/* okano_3_0/HoughLine.cu:1359-1374: ROI-local (angle, distance) to image
 * coordinates, distance += rx*cos(angle) + ry*sin(angle) in float and
 * truncated back to int (host arithmetic, no contraction). */
int HoughLine::getGlobalParam(Image *inimg, int *linesmax, LineParam *lineparam)
{
    if (!inimg || !linesmax || (*linesmax > 0 && !lineparam))
        return NULL_POINTER;
    const int rx = inimg->roiX1, ry = inimg->roiY1;
    if (rx == 0 && ry == 0)
        return NO_ERROR;
    for (int i = 0; i < *linesmax; i++) {
        volatile float a = (float)lineparam[i].distance;
        volatile float b = (float)rx * cosf(lineparam[i].angle);
        volatile float c = (float)ry * sinf(lineparam[i].angle);
        volatile float ab = a + b;
        lineparam[i].distance = (int)(ab + c);
    }
    return NO_ERROR;
}
