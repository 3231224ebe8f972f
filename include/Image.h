/*
 * Image.h -- the 8-bit image container of the drop-in surface.
 *
 * Same records and entry points as okano_3_0/Image.h:44-258 (Image,
 * ImageCuda, IMAGE_CUDA, ImageBasicOp) so HoughLine callers compile
 * unchanged; implemented in opencuda_gb300/csrc/Image.cpp.  Device images are
 * pitched (cudaMallocPitch); deviceId < 0 means host memory.
 */
#ifndef __IMAGE_H__
#define __IMAGE_H__

#include <stddef.h>

#include "ErrorCode.h"

#if defined(__CUDACC__)
#define OCU_HD __host__ __device__
#else
#define OCU_HD
#endif

typedef struct Image_st {
    size_t width;            /* image width, pixels */
    size_t height;           /* image height, pixels */
    int roiX1;               /* ROI [roiX1, roiX2) x [roiY1, roiY2) */
    int roiY1;
    int roiX2;
    int roiY2;
    unsigned char *imgData;  /* pixel (0, 0); host or device memory */
} Image;

typedef struct ImageCuda_st {
    Image imgMeta;           /* must stay the first member (IMAGE_CUDA) */
    int deviceId;            /* -1: host memory, else the CUDA device */
    size_t pitchBytes;       /* bytes per row */
} ImageCuda;

/* Image * -> its enclosing ImageCuda (okano_3_0/Image.h:74-78). */
#define IMAGE_CUDA(img) \
    ((ImageCuda *)((unsigned char *)(img) - offsetof(ImageCuda, imgMeta)))

class ImageBasicOp {
public:
    static int newImage(Image **outimg);
    static int deleteImage(Image *inimg);
    static int makeAtCurrentDevice(Image *img, size_t width, size_t height);
    static int makeAtHost(Image *img, size_t width, size_t height);
    /* 8-bit BMP files (okano_3_0/Image.cu:178-432) */
    static int readFromFile(const char *filepath, Image *outimg);
    static int writeToFile(const char *filepath, Image *inimg);
    /* in-place migration: the image's data moves to the current device /
     * to the host and the old buffer is freed (okano_3_0/Image.cu:435-534) */
    static int copyToCurrentDevice(Image *img);
    static int copyToCurrentDevice(Image *srcimg, Image *dstimg);
    static int copyToHost(Image *img);
    static int copyToHost(Image *srcimg, Image *dstimg);

    /* ROI view as a sub-image (okano_3_0/Image.h:218-258) */
    static OCU_HD int roiSubImage(Image *inimg, ImageCuda *subimgCud)
    {
        if (inimg == NULL || subimgCud == NULL)
            return NULL_POINTER;
        ImageCuda *in = IMAGE_CUDA(inimg);
        if (inimg->imgData == NULL || inimg->width == 0 || inimg->height == 0 ||
            in->pitchBytes == 0)
            return INVALID_DATA;
        subimgCud->imgMeta.width = inimg->roiX2 - inimg->roiX1;
        subimgCud->imgMeta.height = inimg->roiY2 - inimg->roiY1;
        subimgCud->imgMeta.roiX1 = inimg->roiX1;
        subimgCud->imgMeta.roiY1 = inimg->roiY1;
        subimgCud->imgMeta.roiX2 = inimg->roiX2;
        subimgCud->imgMeta.roiY2 = inimg->roiY2;
        subimgCud->imgMeta.imgData = inimg->imgData +
                                     inimg->roiY1 * in->pitchBytes + inimg->roiX1;
        subimgCud->deviceId = in->deviceId;
        subimgCud->pitchBytes = in->pitchBytes;
        return NO_ERROR;
    }
};

#endif
