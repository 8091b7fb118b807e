/* Host program of the --backend cuda path for examples/dot_csv_f.hyd, emitted by codegen_cuda.py.
 * Each fused loop nest is one call into the GB300 runtime (libhyd_cuda.so);
 * procedures return the reference runtime's host arrays. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "hyd_cuda.h"

static double add(double x, double y) {
    return x + y;
}

static double mul(double x, double y) {
    return x * y;
}

static hyd_array_t* a(void) {
    hyd_tuple_t a_shape;
    memset(&a_shape, 0, sizeof a_shape);
    a_shape.ndims = 1;
    a_shape.elems[0] = 3;
    hyd_array_t* a = hyd_cuda_read_float_array_csv("examples/dotA_f.csv", a_shape);
    return a;
}

static hyd_array_t* b(void) {
    hyd_tuple_t b_shape;
    memset(&b_shape, 0, sizeof b_shape);
    b_shape.ndims = 1;
    b_shape.elems[0] = 3;
    hyd_array_t* b = hyd_cuda_read_float_array_csv("examples/dotB_f.csv", b_shape);
    return b;
}

static hyd_array_t* result(void) {
    hyd_array_t* ha = a();
    hyd_array_t* hb = b();
    void* d_a = hyd_cuda_gen_upload(ha);
    void* d_b = hyd_cuda_gen_upload(hb);
    double* d_acc = (double*)hyd_cuda_gen_alloc((int64_t)sizeof(double));
    hyd_cuda_gen_check(hyd_cuda_dot_f64((const double*)d_a, (const double*)d_b, 3, d_acc, NULL), "dot_f64");
    hyd_tuple_t result_shape;
    memset(&result_shape, 0, sizeof result_shape);
    result_shape.ndims = 0;
    hyd_array_t* result = hyd_cuda_gen_download(d_acc, result_shape, sizeof(double));
    hyd_cuda_gen_free(d_a);
    hyd_cuda_gen_free(d_b);
    hyd_cuda_gen_free(d_acc);
    hyd_cuda_gen_array_free(ha);
    hyd_cuda_gen_array_free(hb);
    return result;
}

static double hyd_main(void) {
    hyd_array_t* r = result();
    double v;
    memcpy(&v, r->data, sizeof v);
    hyd_cuda_gen_array_free(r);
    return v;
}

double hyd_export_mul(double x, double y) {
    return mul(x, y);
}

int main(void) {
    hyd_cuda_gen_check(hyd_cuda_init(), "hyd_cuda_init");
    hyd_array_t* a_result = a();
    hyd_cuda_gen_print_float_array(a_result);
    hyd_cuda_gen_array_free(a_result);
    hyd_array_t* b_result = b();
    hyd_cuda_gen_print_float_array(b_result);
    hyd_cuda_gen_array_free(b_result);
    hyd_array_t* result_result = result();
    hyd_cuda_gen_print_float_array(result_result);
    hyd_cuda_gen_array_free(result_result);
    double hyd_main_result = hyd_main();
    hyd_cuda_gen_print_double(hyd_main_result);
    hyd_cuda_cleanup();
    return 0;
}
