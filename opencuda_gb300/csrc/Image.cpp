/*
 * Image.cpp -- ImageBasicOp / TemplateBasicOp of the drop-in surface
 * (include/Image.h, include/Template.h).
 *
 * Semantics follow okano_3_0/Image.cu and okano_3_0/Template.cu: an image or
 * point set lives either on the host (deviceId < 0) or on one CUDA device;
 * copyToCurrentDevice / copyToHost with one argument MIGRATE the object in
 * place (the old buffer is freed -- the reference's visible side effect of
 * HoughLine::houghLine on its input image); with two arguments they copy
 * into the second object.  Device images are pitched (cudaMallocPitch).
 * Errors: NULL_POINTER, INVALID_DATA, UNMATCH_IMG (no data where data is
 * required, okano_3_0/Image.cu:457-460), OP_OVERFLOW (bad device id),
 * CUDA_ERROR, OUT_OF_MEM, NO_FILE, WRONG_FILE.
 */
#include <cuda_runtime.h>

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <new>

#include "CoordiSet.h"
#include "Image.h"

static int cur_device()
{
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

static bool bad_device(int id)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess)
        n = 0;
    return id >= n;
}

/* free an image buffer wherever it lives */
static void free_pixels(unsigned char *p, int dev)
{
    if (!p)
        return;
    if (dev < 0) {
        delete[] p;
        return;
    }
    int cur = cur_device();
    if (dev != cur)
        cudaSetDevice(dev);
    cudaFree(p);
    if (dev != cur)
        cudaSetDevice(cur);
}

int ImageBasicOp::newImage(Image **outimg)
{
    if (!outimg)
        return NULL_POINTER;
    ImageCuda *c = new (std::nothrow) ImageCuda;
    if (!c)
        return OUT_OF_MEM;
    memset(c, 0, sizeof(*c));
    c->deviceId = -1;
    *outimg = &c->imgMeta;
    return NO_ERROR;
}

int ImageBasicOp::deleteImage(Image *inimg)
{
    if (!inimg)
        return NULL_POINTER;
    ImageCuda *c = IMAGE_CUDA(inimg);
    if (bad_device(c->deviceId))
        return OP_OVERFLOW;
    free_pixels(inimg->imgData, c->deviceId);
    delete c;
    return NO_ERROR;
}

int ImageBasicOp::makeAtCurrentDevice(Image *img, size_t width, size_t height)
{
    if (!img)
        return NULL_POINTER;
    if (width < 1 || height < 1)
        return INVALID_DATA;
    if (img->imgData)
        return UNMATCH_IMG;
    ImageCuda *c = IMAGE_CUDA(img);
    size_t pitch = 0;
    if (cudaMallocPitch((void **)&img->imgData, &pitch, width, height) !=
        cudaSuccess) {
        img->imgData = NULL;
        return CUDA_ERROR;
    }
    img->width = width;
    img->height = height;
    img->roiX1 = img->roiY1 = 0;
    img->roiX2 = (int)width;
    img->roiY2 = (int)height;
    c->deviceId = cur_device();
    c->pitchBytes = pitch;
    return NO_ERROR;
}

int ImageBasicOp::makeAtHost(Image *img, size_t width, size_t height)
{
    if (!img)
        return NULL_POINTER;
    if (width < 1 || height < 1)
        return INVALID_DATA;
    if (img->imgData)
        return UNMATCH_IMG;
    ImageCuda *c = IMAGE_CUDA(img);
    img->imgData = new (std::nothrow) unsigned char[width * height];
    if (!img->imgData)
        return OUT_OF_MEM;
    img->width = width;
    img->height = height;
    img->roiX1 = img->roiY1 = 0;
    img->roiX2 = (int)width;
    img->roiY2 = (int)height;
    c->deviceId = -1;
    c->pitchBytes = width;
    return NO_ERROR;
}

static bool has_pixels(const Image *img)
{
    const ImageCuda *c = IMAGE_CUDA(const_cast<Image *>(img));
    return img->imgData && img->width && img->height && c->pitchBytes;
}

int ImageBasicOp::copyToCurrentDevice(Image *img)
{
    if (!img)
        return NULL_POINTER;
    ImageCuda *c = IMAGE_CUDA(img);
    if (bad_device(c->deviceId))
        return OP_OVERFLOW;
    if (!has_pixels(img))
        return UNMATCH_IMG;
    const int cur = cur_device();
    if (c->deviceId == cur)
        return NO_ERROR;
    unsigned char *dst = NULL;
    size_t pitch = 0;
    if (cudaMallocPitch((void **)&dst, &pitch, img->width, img->height) !=
        cudaSuccess)
        return CUDA_ERROR;
    cudaError_t e;
    if (c->deviceId < 0)
        e = cudaMemcpy2D(dst, pitch, img->imgData, c->pitchBytes, img->width,
                         img->height, cudaMemcpyHostToDevice);
    else   /* another device: peer copy row block by row block */
        e = cudaMemcpy2D(dst, pitch, img->imgData, c->pitchBytes, img->width,
                         img->height, cudaMemcpyDefault);
    if (e != cudaSuccess) {
        cudaFree(dst);
        return CUDA_ERROR;
    }
    free_pixels(img->imgData, c->deviceId);
    img->imgData = dst;
    c->deviceId = cur;
    c->pitchBytes = pitch;
    return NO_ERROR;
}

int ImageBasicOp::copyToHost(Image *img)
{
    if (!img)
        return NULL_POINTER;
    ImageCuda *c = IMAGE_CUDA(img);
    if (bad_device(c->deviceId))
        return OP_OVERFLOW;
    if (!has_pixels(img))
        return UNMATCH_IMG;
    if (c->deviceId < 0)
        return NO_ERROR;
    unsigned char *dst = new (std::nothrow) unsigned char[img->width * img->height];
    if (!dst)
        return OUT_OF_MEM;
    if (cudaMemcpy2D(dst, img->width, img->imgData, c->pitchBytes, img->width,
                     img->height, cudaMemcpyDefault) != cudaSuccess) {
        delete[] dst;
        return CUDA_ERROR;
    }
    free_pixels(img->imgData, c->deviceId);
    img->imgData = dst;
    c->deviceId = -1;
    c->pitchBytes = img->width;
    return NO_ERROR;
}

/* copy src into dst, giving dst a fresh buffer on `dev` (-1 host) unless
 * its current one already fits */
static int copy_into(Image *src, Image *dst, int dev)
{
    if (!src)
        return NULL_POINTER;
    ImageCuda *sc = IMAGE_CUDA(src), *dc = IMAGE_CUDA(dst);
    if (!has_pixels(src))
        return INVALID_DATA;
    if (bad_device(sc->deviceId) || bad_device(dc->deviceId))
        return OP_OVERFLOW;
    bool reuse = dst->imgData && dc->deviceId == dev &&
                 dst->width == src->width && dst->height == src->height;
    unsigned char *buf = reuse ? dst->imgData : NULL;
    size_t pitch = reuse ? dc->pitchBytes : 0;
    if (!reuse) {
        if (dev < 0) {
            buf = new (std::nothrow) unsigned char[src->width * src->height];
            if (!buf)
                return OUT_OF_MEM;
            pitch = src->width;
        } else if (cudaMallocPitch((void **)&buf, &pitch, src->width,
                                   src->height) != cudaSuccess) {
            return CUDA_ERROR;
        }
    }
    if (cudaMemcpy2D(buf, pitch, src->imgData, sc->pitchBytes, src->width,
                     src->height, cudaMemcpyDefault) != cudaSuccess) {
        if (!reuse)
            free_pixels(buf, dev);
        return CUDA_ERROR;
    }
    if (!reuse)
        free_pixels(dst->imgData, dc->deviceId);
    dst->imgData = buf;
    dst->width = src->width;
    dst->height = src->height;
    dst->roiX1 = src->roiX1;
    dst->roiY1 = src->roiY1;
    dst->roiX2 = src->roiX2;
    dst->roiY2 = src->roiY2;
    dc->deviceId = dev;
    dc->pitchBytes = pitch;
    return NO_ERROR;
}

int ImageBasicOp::copyToCurrentDevice(Image *srcimg, Image *dstimg)
{
    if (!srcimg)
        return NULL_POINTER;
    if (!dstimg || dstimg == srcimg)
        return copyToCurrentDevice(srcimg);
    return copy_into(srcimg, dstimg, cur_device());
}

int ImageBasicOp::copyToHost(Image *srcimg, Image *dstimg)
{
    if (!srcimg)
        return NULL_POINTER;
    if (!dstimg || dstimg == srcimg)
        return copyToHost(srcimg);
    return copy_into(srcimg, dstimg, -1);
}

/* 8-bit palette BMP, bottom-up rows padded to 4 bytes
 * (okano_3_0/Image.cu:178-432). */
static unsigned rd32(const unsigned char *p)
{
    return p[0] | (p[1] << 8) | (p[2] << 16) | ((unsigned)p[3] << 24);
}

int ImageBasicOp::readFromFile(const char *filepath, Image *outimg)
{
    if (!filepath || !outimg)
        return NULL_POINTER;
    ImageCuda *c = IMAGE_CUDA(outimg);
    if (bad_device(c->deviceId))
        return OP_OVERFLOW;
    FILE *f = fopen(filepath, "rb");
    if (!f)
        return NO_FILE;
    unsigned char hdr[54];
    if (fread(hdr, 1, 54, f) != 54 || hdr[0] != 'B' || hdr[1] != 'M' ||
        (hdr[28] | (hdr[29] << 8)) != 8) {
        fclose(f);
        return WRONG_FILE;
    }
    unsigned w = rd32(hdr + 18), h = rd32(hdr + 22), off = rd32(hdr + 10);
    if (w < 1 || h < 1 || (int)h < 0) {
        fclose(f);
        return WRONG_FILE;
    }
    unsigned char *buf = new (std::nothrow) unsigned char[(size_t)w * h];
    if (!buf) {
        fclose(f);
        return OUT_OF_MEM;
    }
    const unsigned pad = (4 - (w & 3)) & 3;
    fseek(f, (long)off, SEEK_SET);
    for (unsigned r = 0; r < h; r++) {
        unsigned char *row = buf + (size_t)(h - 1 - r) * w;
        if (fread(row, 1, w, f) != w) {
            delete[] buf;
            fclose(f);
            return WRONG_FILE;
        }
        if (pad)
            fseek(f, (long)pad, SEEK_CUR);
    }
    fclose(f);
    free_pixels(outimg->imgData, c->deviceId);
    outimg->imgData = buf;
    outimg->width = w;
    outimg->height = h;
    outimg->roiX1 = outimg->roiY1 = 0;
    outimg->roiX2 = (int)w;
    outimg->roiY2 = (int)h;
    c->deviceId = -1;
    c->pitchBytes = w;
    return NO_ERROR;
}

static void wr32(unsigned char *p, unsigned v)
{
    p[0] = v & 255;
    p[1] = (v >> 8) & 255;
    p[2] = (v >> 16) & 255;
    p[3] = v >> 24;
}

int ImageBasicOp::writeToFile(const char *filepath, Image *inimg)
{
    if (!filepath || !inimg)
        return NULL_POINTER;
    int rc = copyToHost(inimg);   /* the reference migrates to the host too */
    if (rc < 0)
        return rc;
    FILE *f = fopen(filepath, "wb");
    if (!f)
        return NO_FILE;
    ImageCuda *c = IMAGE_CUDA(inimg);
    const unsigned w = (unsigned)inimg->width, h = (unsigned)inimg->height;
    const unsigned pad = (4 - (w & 3)) & 3;
    const unsigned datalen = h * (w + pad), off = 54 + 4 * 256;
    unsigned char hdr[54];
    memset(hdr, 0, sizeof(hdr));
    hdr[0] = 'B';
    hdr[1] = 'M';
    wr32(hdr + 2, off + datalen);
    wr32(hdr + 10, off);
    wr32(hdr + 14, 40);
    wr32(hdr + 18, w);
    wr32(hdr + 22, h);
    hdr[26] = 1;
    hdr[28] = 8;
    wr32(hdr + 34, datalen);
    wr32(hdr + 46, 256);
    fwrite(hdr, 1, 54, f);
    for (int i = 0; i < 256; i++) {
        unsigned char q[4] = {(unsigned char)i, (unsigned char)i, (unsigned char)i, 0xFF};
        fwrite(q, 1, 4, f);
    }
    const unsigned char zero[4] = {0, 0, 0, 0};
    for (unsigned r = 0; r < h; r++) {
        fwrite(inimg->imgData + (size_t)(h - 1 - r) * c->pitchBytes, 1, w, f);
        if (pad)
            fwrite(zero, 1, pad, f);
    }
    fclose(f);
    return NO_ERROR;
}

/* ---------------------------------------------------------------------- */
/* Template / CoordiSet                                                     */

static void free_points(Template *t, TemplateCuda *c)
{
    if (c->deviceId < 0) {
        delete[] t->tplData;
        delete[] c->attachedData;
    } else {
        int cur = cur_device();
        if (c->deviceId != cur)
            cudaSetDevice(c->deviceId);
        cudaFree(t->tplData);
        cudaFree(c->attachedData);
        if (c->deviceId != cur)
            cudaSetDevice(cur);
    }
    t->tplData = NULL;
    c->attachedData = NULL;
}

int TemplateBasicOp::newTemplate(Template **outtpl)
{
    if (!outtpl)
        return NULL_POINTER;
    TemplateCuda *c = new (std::nothrow) TemplateCuda;
    if (!c)
        return OUT_OF_MEM;
    memset(c, 0, sizeof(*c));
    c->deviceId = -1;
    *outtpl = &c->tplMeta;
    return NO_ERROR;
}

int TemplateBasicOp::deleteTemplate(Template *intpl)
{
    if (!intpl)
        return NULL_POINTER;
    TemplateCuda *c = TEMPLATE_CUDA(intpl);
    if (bad_device(c->deviceId))
        return OP_OVERFLOW;
    free_points(intpl, c);
    delete c;
    return NO_ERROR;
}

int TemplateBasicOp::makeAtCurrentDevice(Template *tpl, size_t count)
{
    if (!tpl)
        return NULL_POINTER;
    if (count < 1)
        return INVALID_DATA;
    if (tpl->tplData)
        return UNMATCH_IMG;
    TemplateCuda *c = TEMPLATE_CUDA(tpl);
    if (cudaMalloc((void **)&tpl->tplData, sizeof(int) * 2 * count) != cudaSuccess)
        return CUDA_ERROR;
    if (cudaMalloc((void **)&c->attachedData, sizeof(float) * count) != cudaSuccess) {
        cudaFree(tpl->tplData);
        tpl->tplData = NULL;
        return CUDA_ERROR;
    }
    tpl->count = count;
    c->deviceId = cur_device();
    return NO_ERROR;
}

int TemplateBasicOp::makeAtHost(Template *tpl, size_t count)
{
    if (!tpl)
        return NULL_POINTER;
    if (count < 1)
        return INVALID_DATA;
    if (tpl->tplData)
        return UNMATCH_IMG;
    TemplateCuda *c = TEMPLATE_CUDA(tpl);
    tpl->tplData = new (std::nothrow) int[2 * count];
    c->attachedData = new (std::nothrow) float[count];
    if (!tpl->tplData || !c->attachedData) {
        delete[] tpl->tplData;
        delete[] c->attachedData;
        tpl->tplData = NULL;
        c->attachedData = NULL;
        return OUT_OF_MEM;
    }
    tpl->count = count;
    c->deviceId = -1;
    return NO_ERROR;
}

static int move_points(Template *tpl, int dev)
{
    TemplateCuda *c = TEMPLATE_CUDA(tpl);
    if (bad_device(c->deviceId))
        return OP_OVERFLOW;
    if (!tpl->tplData || tpl->count == 0)
        return UNMATCH_IMG;
    if (c->deviceId == dev)
        return NO_ERROR;
    const size_t n = tpl->count;
    int *xy = NULL;
    float *att = NULL;
    if (dev < 0) {
        xy = new (std::nothrow) int[2 * n];
        att = new (std::nothrow) float[n];
        if (!xy || !att) {
            delete[] xy;
            delete[] att;
            return OUT_OF_MEM;
        }
    } else if (cudaMalloc((void **)&xy, sizeof(int) * 2 * n) != cudaSuccess ||
               cudaMalloc((void **)&att, sizeof(float) * n) != cudaSuccess) {
        cudaFree(xy);
        return CUDA_ERROR;
    }
    cudaError_t e = cudaMemcpy(xy, tpl->tplData, sizeof(int) * 2 * n, cudaMemcpyDefault);
    if (e == cudaSuccess && c->attachedData)
        e = cudaMemcpy(att, c->attachedData, sizeof(float) * n, cudaMemcpyDefault);
    if (e != cudaSuccess) {
        if (dev < 0) {
            delete[] xy;
            delete[] att;
        } else {
            cudaFree(xy);
            cudaFree(att);
        }
        return CUDA_ERROR;
    }
    free_points(tpl, c);
    tpl->tplData = xy;
    c->attachedData = att;
    c->deviceId = dev;
    return NO_ERROR;
}

int TemplateBasicOp::copyToCurrentDevice(Template *tpl)
{
    if (!tpl)
        return NULL_POINTER;
    return move_points(tpl, cur_device());
}

int TemplateBasicOp::copyToHost(Template *tpl)
{
    if (!tpl)
        return NULL_POINTER;
    return move_points(tpl, -1);
}

static int copy_points(Template *src, Template *dst, int dev)
{
    if (!src)
        return NULL_POINTER;
    if (!dst || dst == src)
        return move_points(src, dev);
    if (!src->tplData || src->count == 0)
        return INVALID_DATA;
    TemplateCuda *sc = TEMPLATE_CUDA(src), *dc = TEMPLATE_CUDA(dst);
    free_points(dst, dc);
    dst->count = 0;
    dc->deviceId = dev;
    int rc = (dev < 0) ? TemplateBasicOp::makeAtHost(dst, src->count)
                       : TemplateBasicOp::makeAtCurrentDevice(dst, src->count);
    if (rc != NO_ERROR)
        return rc;
    if (cudaMemcpy(dst->tplData, src->tplData, sizeof(int) * 2 * src->count,
                   cudaMemcpyDefault) != cudaSuccess)
        return CUDA_ERROR;
    if (sc->attachedData &&
        cudaMemcpy(dc->attachedData, sc->attachedData, sizeof(float) * src->count,
                   cudaMemcpyDefault) != cudaSuccess)
        return CUDA_ERROR;
    return NO_ERROR;
}

int TemplateBasicOp::copyToCurrentDevice(Template *srctpl, Template *dsttpl)
{
    return copy_points(srctpl, dsttpl, cur_device());
}

int TemplateBasicOp::copyToHost(Template *srctpl, Template *dsttpl)
{
    return copy_points(srctpl, dsttpl, -1);
}

int TemplateBasicOp::readFromFile(const char *filepath, Template *outtpl)
{
    if (!filepath || !outtpl)
        return NULL_POINTER;
    FILE *f = fopen(filepath, "r");
    if (!f)
        return NO_FILE;
    long n = 0;
    if (fscanf(f, "%ld", &n) != 1 || n < 1) {
        fclose(f);
        return WRONG_FILE;
    }
    TemplateCuda *c = TEMPLATE_CUDA(outtpl);
    free_points(outtpl, c);
    outtpl->count = 0;
    int rc = makeAtHost(outtpl, (size_t)n);
    if (rc != NO_ERROR) {
        fclose(f);
        return rc;
    }
    for (long i = 0; i < n; i++) {
        if (fscanf(f, "%d %d %f", &outtpl->tplData[2 * i], &outtpl->tplData[2 * i + 1],
                   &c->attachedData[i]) != 3) {
            fclose(f);
            return WRONG_FILE;
        }
    }
    fclose(f);
    return NO_ERROR;
}

int TemplateBasicOp::writeToFile(const char *filepath, Template *intpl)
{
    if (!filepath || !intpl)
        return NULL_POINTER;
    int rc = copyToHost(intpl);
    if (rc != NO_ERROR)
        return rc;
    FILE *f = fopen(filepath, "w");
    if (!f)
        return NO_FILE;
    TemplateCuda *c = TEMPLATE_CUDA(intpl);
    fprintf(f, "%zu\n", intpl->count);
    for (size_t i = 0; i < intpl->count; i++)
        fprintf(f, "%d %d %.9g\n", intpl->tplData[2 * i], intpl->tplData[2 * i + 1],
                c->attachedData ? c->attachedData[i] : 0.0f);
    fclose(f);
    return NO_ERROR;
}
