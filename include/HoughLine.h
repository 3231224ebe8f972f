/*
 * HoughLine.h -- drop-in replacement for OpenCUDA's HoughLine class
 * (okano_3_0/HoughLine.h:82-330): same members, defaults, signatures and
 * ErrorCode returns; the work runs on the GB300 kernels of
 * libhoughline_gb300.so through its C ABI (houghline_gb300.h).
 *
 * Differences a caller can see (all documented in the implementation):
 *   - ties between equal vote counts are ranked by bin index (rho-major,
 *     theta-minor) instead of the reference's unstable Shell sort order;
 *   - the coordinate-set accumulator covers every input point, so sets far
 *     from the origin no longer index outside the accumulator;
 *   - an empty ROI returns INVALID_DATA (the reference launched an empty
 *     grid and returned CUDA_ERROR);
 *   - realLine returns false on a CUDA failure (the reference returned the
 *     error code converted to bool).
 * The object keeps a GPU workspace that is created on first use and reused
 * by later calls; copies of a HoughLine get their own workspace.
 */
#ifndef __HOUGHLINE_H__
#define __HOUGHLINE_H__

#include <math.h>

#include "CoordiSet.h"
#include "ErrorCode.h"
#include "Image.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* okano_3_0/HoughLine.h:70-74 */
typedef struct LineParam_st {
    float angle;    /* radians */
    int distance;   /* rho */
    int votes;      /* accumulator count */
} LineParam;

struct hl_handle;

class HoughLine {
protected:
    double detheta;    /* angle step, radians */
    double derho;      /* distance step */
    int threshold;     /* peak threshold (votes > threshold) */
    float thresang;    /* merge angle, radians */
    int thresdis;      /* merge distance */

private:
    mutable struct hl_handle *gpu_;   /* GB300 workspace, created lazily */
    int sync_params() const;

public:
    /* okano_3_0/HoughLine.h:116-125 */
    HoughLine()
        : detheta(M_PI / 180), derho(1.0), threshold(90),
          thresang((float)(M_PI / 180 * 5.0f)), thresdis(50), gpu_(NULL)
    {
    }

    /* okano_3_0/HoughLine.h:129-156 */
    HoughLine(double detheta, double derho, int threshold, float thresang,
              int thresdis)
        : detheta(M_PI / 180), derho(1.0), threshold(90),
          thresang((float)(M_PI / 180 * 5.0)), thresdis(50), gpu_(NULL)
    {
        setDeTheta(detheta);
        setDeRho(derho);
        setThreshold(threshold);
        setThresAng(thresang);
        setThresDis(thresdis);
    }

    HoughLine(const HoughLine &o)
        : detheta(o.detheta), derho(o.derho), threshold(o.threshold),
          thresang(o.thresang), thresdis(o.thresdis), gpu_(NULL)
    {
    }
    HoughLine &operator=(const HoughLine &o);
    ~HoughLine();

    double getDeTheta() const { return detheta; }
    int setDeTheta(double v) { detheta = v; return NO_ERROR; }
    double getDeRho() const { return derho; }
    int setDeRho(double v) { derho = v; return NO_ERROR; }
    int getThreshold() const { return threshold; }
    int setThreshold(int v) { threshold = v; return NO_ERROR; }
    float getThresAng() const { return thresang; }
    int setThresAng(float v) { thresang = v; return NO_ERROR; }
    int getThresDis() const { return thresdis; }
    int setThresDis(int v) { thresdis = v; return NO_ERROR; }

    /* okano_3_0/HoughLine.cu:352-632 */
    int houghLineCor(CoordiSet *guidingset, int *linesmax,
                     LineParam *lineparam);
    /* okano_3_0/HoughLine.cu:635-955 */
    int houghLine(Image *inimg, CoordiSet *guidingset, int *linesmax,
                  LineParam *lineparam);
    /* okano_3_0/HoughLine.cu:958-1345 */
    int houghLineImg(Image *inimg, CoordiSet *guidingset, Image *outimg,
                     int *linesmax, LineParam *lineparam);
    /* okano_3_0/HoughLine.cu:1377-1462 */
    bool realLine(Image *inimg, int x1, int y1, int x2, int y2,
                  float threshold, float thresperc);
    /* okano_3_0/HoughLine.cu:1359-1374 */
    int getGlobalParam(Image *inimg, int *linesmax, LineParam *lineparam);
};

#endif
