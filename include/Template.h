/*
 * Template.h -- point-set container of the drop-in surface (the storage of
 * CoordiSet).  Same records and entry points as okano_3_0/Template.h:14-180:
 * tplData holds count interleaved (x, y) ints; attachedData one float per
 * point; deviceId < 0 means host memory.  Implemented in
 * opencuda_gb300/csrc/Image.cpp.
 */
#ifndef __TEMPLATE_H__
#define __TEMPLATE_H__

#include <stddef.h>

#include "ErrorCode.h"

typedef struct Template_st {
    size_t count;    /* number of points */
    int *tplData;    /* x0, y0, x1, y1, ... */
} Template;

typedef struct TemplateCuda_st {
    Template tplMeta;     /* must stay the first member (TEMPLATE_CUDA) */
    float *attachedData;  /* count floats, same memory space as tplData */
    int deviceId;         /* -1: host memory, else the CUDA device */
} TemplateCuda;

#define TEMPLATE_CUDA(tpl) \
    ((TemplateCuda *)((unsigned char *)(tpl) - offsetof(TemplateCuda, tplMeta)))
#define ATTACHED_DATA(tpl) (TEMPLATE_CUDA(tpl)->attachedData)

class TemplateBasicOp {
public:
    static int newTemplate(Template **outtpl);
    static int deleteTemplate(Template *intpl);
    static int makeAtCurrentDevice(Template *tpl, size_t count);
    static int makeAtHost(Template *tpl, size_t count);
    /* plain text: count, then one "x y attached" line per point */
    static int readFromFile(const char *filepath, Template *outtpl);
    static int writeToFile(const char *filepath, Template *intpl);
    static int copyToCurrentDevice(Template *tpl);
    static int copyToCurrentDevice(Template *srctpl, Template *dsttpl);
    static int copyToHost(Template *tpl);
    static int copyToHost(Template *srctpl, Template *dsttpl);
};

#endif
