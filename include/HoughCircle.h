/*
 * HoughCircle.h -- drop-in replacement for OpenCUDA's HoughCircle class
 * (okano_3_0/HoughCircle.h:37-254): same members, defaults, setters,
 * signatures and ErrorCode returns; the work runs on the GB300 circle kernels
 * of libhoughline_gb300.so through its C ABI (hl_circle.h).
 *
 * Differences a caller can see:
 *   - circles with equal votes are ranked by (radius, row, column) index
 *     instead of the order the reference's shear sort leaves them in;
 *   - writetofile draws nothing, and no result.bmp is written (the reference
 *     writes that file on every houghcircle call);
 *   - more than 4096 local maxima above cirThreshold return OP_OVERFLOW;
 *   - pieceCircle returns the first error of a piece (the reference ignores
 *     it and copies the piece's unset records).
 * The object keeps a GPU workspace that is created on first use and reused
 * by later calls; copies of a HoughCircle get their own workspace.
 */
#ifndef __HOUGHCIRCLE_H__
#define __HOUGHCIRCLE_H__

#include "CoordiSet.h"
#include "ErrorCode.h"
#include "Image.h"

/* okano_3_0/HoughCircle.h:41-46 */
typedef struct CircleParam_st {
    int a;        /* centre column */
    int b;        /* centre row */
    int radius;
    int votes;
} CircleParam;

struct hl_handle;

class HoughCircle {
protected:
    int radiusMin;
    int radiusMax;
    float distThres;
    float rThres;
    int cirThreshold;

private:
    mutable struct hl_handle *gpu_;   /* GB300 workspace, created lazily */
    int ensure() const;

public:
    /* okano_3_0/HoughCircle.h:79-90 */
    HoughCircle()
        : radiusMin(5), radiusMax(50), distThres(50.0f), rThres(20), cirThreshold(100),
          gpu_(NULL)
    {
    }

    /* okano_3_0/HoughCircle.h:93-115: defaults first, then the setters (an
     * invalid value keeps the default) */
    HoughCircle(int radiusMin, int radiusMax, float distMin, int rThres, int cirThreshold)
        : radiusMin(5), radiusMax(50), distThres(50.0f), rThres(20), cirThreshold(100),
          gpu_(NULL)
    {
        setRadiusMin(radiusMin);
        setRadiusMax(radiusMax);
        setDistThres(distMin);
        setRThres(rThres);
        setCirThreshold(cirThreshold);
    }

    HoughCircle(const HoughCircle &o)
        : radiusMin(o.radiusMin), radiusMax(o.radiusMax), distThres(o.distThres),
          rThres(o.rThres), cirThreshold(o.cirThreshold), gpu_(NULL)
    {
    }
    HoughCircle &operator=(const HoughCircle &o);
    ~HoughCircle();

    int getRadiusMin() const { return radiusMin; }
    int setRadiusMin(int v)
    {
        if (v < 0)
            return INVALID_DATA;
        radiusMin = v;
        return NO_ERROR;
    }
    int getRadiusMax() const { return radiusMax; }
    int setRadiusMax(int v)
    {
        if (v < 0)
            return INVALID_DATA;
        radiusMax = v;
        return NO_ERROR;
    }
    float getDistThres() const { return distThres; }
    int setDistThres(float v)
    {
        distThres = v;
        return NO_ERROR;
    }
    int getRThres() const { return (int)rThres; }
    int setRThres(int v)
    {
        rThres = (float)v;
        return NO_ERROR;
    }
    int getCirThreshold() const { return cirThreshold; }
    int setCirThreshold(int v)
    {
        if (v < 0)
            return INVALID_DATA;
        cirThreshold = v;
        return NO_ERROR;
    }

    /* okano_3_0/HoughCircle.cu:1236-1320: the circles of the image's ROI
     * (centres in image coordinates), or of a point set drawn into a
     * (max x + 2) x (max y + 2) image; *circleMax in (room) / out (found) */
    int houghcircle(Image *inimg, CoordiSet *guidingset, int *circleMax,
                    CircleParam *circleparam, bool writetofile);
    /* okano_3_0/HoughCircle.cu:1323-1400: piecenum x piecenum pieces of
     * (width / piecenum) x (height / piecenum), ROI [x * c, x * c + c - 1),
     * up to 10 circles each, concatenated in row-major piece order */
    int pieceCircle(Image *inimg, int piecenum, int *circleMax, CircleParam *circleparam,
                    bool writetofile);
};

#endif
