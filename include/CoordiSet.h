/*
 * CoordiSet.h -- coordinate set = Template (okano_3_0/CoordiSet.h:15-43),
 * with CoordiSetBasicOp forwarding to TemplateBasicOp.
 */
#ifndef __COORDISET_H__
#define __COORDISET_H__

#include "Template.h"

typedef Template CoordiSet;
typedef TemplateCuda CoordiSetCuda;
#define COORDISET_CUDA(cst) TEMPLATE_CUDA(cst)

class CoordiSetBasicOp {
public:
    static inline int newCoordiSet(CoordiSet **outcst)
    { return TemplateBasicOp::newTemplate(outcst); }
    static inline int deleteCoordiSet(CoordiSet *incst)
    { return TemplateBasicOp::deleteTemplate(incst); }
    static inline int makeAtCurrentDevice(CoordiSet *cst, size_t count)
    { return TemplateBasicOp::makeAtCurrentDevice(cst, count); }
    static inline int makeAtHost(CoordiSet *cst, size_t count)
    { return TemplateBasicOp::makeAtHost(cst, count); }
    static inline int readFromFile(const char *filepath, CoordiSet *outcst)
    { return TemplateBasicOp::readFromFile(filepath, outcst); }
    static inline int writeToFile(const char *filepath, CoordiSet *incst)
    { return TemplateBasicOp::writeToFile(filepath, incst); }
    static inline int copyToCurrentDevice(CoordiSet *cst)
    { return TemplateBasicOp::copyToCurrentDevice(cst); }
    static inline int copyToCurrentDevice(CoordiSet *src, CoordiSet *dst)
    { return TemplateBasicOp::copyToCurrentDevice(src, dst); }
    static inline int copyToHost(CoordiSet *cst)
    { return TemplateBasicOp::copyToHost(cst); }
    static inline int copyToHost(CoordiSet *src, CoordiSet *dst)
    { return TemplateBasicOp::copyToHost(src, dst); }
};

#endif
