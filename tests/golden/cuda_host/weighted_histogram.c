/* Host program of the --backend cuda path for examples/weighted_histogram.hyd, emitted by codegen_cuda.py.
 * Each fused loop nest is one call into the GB300 runtime (libhyd_cuda.so);
 * procedures return the reference runtime's host arrays. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "hyd_cuda.h"

static hyd_array_t* data(void) {
    int64_t* d_data = (int64_t*)hyd_cuda_gen_alloc((1024) * (int64_t)sizeof(int64_t));
    {
        hyd_cuda_gen_check(hyd_cuda_map_i64("v = i;", NULL, 0, 1024, d_data, NULL, NULL), "map_i64");
    }
    hyd_tuple_t data_shape;
    memset(&data_shape, 0, sizeof data_shape);
    data_shape.ndims = 1;
    data_shape.elems[0] = 1024;
    hyd_array_t* data = hyd_cuda_gen_download(d_data, data_shape, sizeof(int64_t));
    hyd_cuda_gen_free(d_data);
    return data;
}

static int64_t binFn(int64_t x) {
    return x % 64;
}

static int64_t valueFn(int64_t x) {
    return x * x;
}

static hyd_array_t* hyd_main(void) {
    int64_t* d_data = (int64_t*)hyd_cuda_gen_alloc((1024) * (int64_t)sizeof(int64_t));
    {
        hyd_cuda_gen_check(hyd_cuda_map_i64("v = i;", NULL, 0, 1024, d_data, NULL, NULL), "map_i64");
    }
    int64_t* d_hist = (int64_t*)hyd_cuda_gen_alloc(64LL * (int64_t)sizeof(int64_t));
    hyd_cuda_gen_zero(d_hist, 64LL * (int64_t)sizeof(int64_t));
    hyd_cuda_gen_check(hyd_cuda_weighted_histogram_i64(d_data, 1024, 64LL, d_hist, HYD_SCATTER_AUTO, NULL), "scatter (+)");
    hyd_tuple_t hist_shape;
    memset(&hist_shape, 0, sizeof hist_shape);
    hist_shape.ndims = 1;
    hist_shape.elems[0] = 64;
    hyd_array_t* hist = hyd_cuda_gen_download(d_hist, hist_shape, sizeof(int64_t));
    hyd_cuda_gen_free(d_data);
    hyd_cuda_gen_free(d_hist);
    return hist;
}

int64_t hyd_export_binFn(int64_t x) {
    return binFn(x);
}

int main(void) {
    hyd_cuda_gen_check(hyd_cuda_init(), "hyd_cuda_init");
    hyd_array_t* data_result = data();
    hyd_cuda_gen_print_array(data_result);
    hyd_cuda_gen_array_free(data_result);
    hyd_array_t* hyd_main_result = hyd_main();
    hyd_cuda_gen_print_array(hyd_main_result);
    hyd_cuda_gen_array_free(hyd_main_result);
    hyd_cuda_cleanup();
    return 0;
}
