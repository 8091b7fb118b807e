#ifndef HYDRANGEA_EXPORT_MUL_H
#define HYDRANGEA_EXPORT_MUL_H

#include "hyd_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

double hyd_export_mul(double x, double y);

#ifdef __cplusplus
}
#endif

#endif
