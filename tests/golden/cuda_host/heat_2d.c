/* Host program of the --backend cuda path for examples/heat_2d.hyd, emitted by codegen_cuda.py.
 * Each fused loop nest is one call into the GB300 runtime (libhyd_cuda.so);
 * procedures return the reference runtime's host arrays. */
/* main's result array is released after the write, as the C backend's main does not print it */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "hyd_cuda.h"

static int64_t n(void) {
    int64_t v = 8LL;
    return v;
}

static int64_t iters(void) {
    int64_t v = 4LL;
    return v;
}

static hyd_array_t* init(void) {
    int64_t nn = n();
    double* d_init = (double*)hyd_cuda_gen_alloc((nn * nn) * (int64_t)sizeof(double));
    {
        char body[512];
        snprintf(body, sizeof body, "long long r = i / %lld; long long c = i %% %lld; v = (double)((r * 8) + c) * 0.01;", (long long)nn, (long long)nn);
        hyd_cuda_gen_check(hyd_cuda_map_f64(body, NULL, 0, nn * nn, d_init, NULL, NULL), "map_f64");
    }
    hyd_tuple_t init_shape;
    memset(&init_shape, 0, sizeof init_shape);
    init_shape.ndims = 2;
    init_shape.elems[0] = nn;
    init_shape.elems[1] = nn;
    hyd_array_t* init = hyd_cuda_gen_download(d_init, init_shape, sizeof(double));
    hyd_cuda_gen_free(d_init);
    return init;
}

static hyd_array_t* result(void) {
    int64_t nn = n();
    int64_t k = iters();
    hyd_array_t* h0 = init();
    void* d0 = hyd_cuda_gen_upload(h0);
    double* d_res_pong = (double*)hyd_cuda_gen_alloc((nn) * (nn) * (int64_t)sizeof(double));
    double* d_res;
    {
        int final_buf = 0;
        hyd_cuda_gen_check(hyd_cuda_iterate_stencil2d_f64(HYD_STENCIL_HEAT_EXAMPLE, (double*)d0, d_res_pong, nn, nn, k, &final_buf, NULL), "iterate");
        d_res = final_buf ? d_res_pong : (double*)d0;
    }
    hyd_tuple_t result_shape;
    memset(&result_shape, 0, sizeof result_shape);
    result_shape.ndims = 2;
    result_shape.elems[0] = nn;
    result_shape.elems[1] = nn;
    hyd_array_t* result = hyd_cuda_gen_download(d_res, result_shape, sizeof(double));
    hyd_cuda_gen_free(d0);
    hyd_cuda_gen_free(d_res_pong);
    hyd_cuda_gen_array_free(h0);
    return result;
}

static int64_t hyd_main(void) {
    hyd_array_t* r = result();
    int64_t written = hyd_cuda_write_array_csv_float(r, "heat_2d_out.csv");
    hyd_cuda_gen_array_free(r);
    return written;
}

int main(void) {
    hyd_cuda_gen_check(hyd_cuda_init(), "hyd_cuda_init");
    int64_t n_result = n();
    hyd_cuda_gen_print_int(n_result);
    int64_t iters_result = iters();
    hyd_cuda_gen_print_int(iters_result);
    hyd_array_t* init_result = init();
    hyd_cuda_gen_print_float_array(init_result);
    hyd_cuda_gen_array_free(init_result);
    hyd_array_t* result_result = result();
    hyd_cuda_gen_print_float_array(result_result);
    hyd_cuda_gen_array_free(result_result);
    int64_t hyd_main_result = hyd_main();
    hyd_cuda_gen_print_int(hyd_main_result);
    hyd_cuda_cleanup();
    return 0;
}
