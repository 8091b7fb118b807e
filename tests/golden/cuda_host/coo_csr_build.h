#ifndef HYDRANGEA_EXPORT_IMOD_H
#define HYDRANGEA_EXPORT_IMOD_H

#include "hyd_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

int64_t hyd_export_imod(int64_t x, int64_t m);

#ifdef __cplusplus
}
#endif

#endif
