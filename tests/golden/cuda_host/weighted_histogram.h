#ifndef HYDRANGEA_EXPORT_BINFN_H
#define HYDRANGEA_EXPORT_BINFN_H

#include "hyd_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

int64_t hyd_export_binFn(int64_t x);

#ifdef __cplusplus
}
#endif

#endif
