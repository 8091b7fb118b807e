/* Witness: the reference runtime's CSV input (hyd_read_array_csv and
 * hyd_read_float_array_csv, runtime/hydrangea_runtime.h:549-592) and output
 * (runtime/hyd_write_csv.c, which also defines getenv_int / getenv_string),
 * compiled unmodified.  Their failures call exit(1), as in the reference.
 * TEST INFRASTRUCTURE ONLY. */
#include <stdint.h>
#include <string.h>
#include "runtime/hyd_write_csv.c"

static hyd_tuple_t wit_shape(int ndims, int64_t d0, int64_t d1) {
    hyd_tuple_t s;
    memset(&s, 0, sizeof s);
    s.ndims = ndims;
    s.elems[0] = d0;
    s.elems[1] = d1;
    return s;
}

void wit_read_array_csv(const char* path, int64_t n, int64_t* out) {
    hyd_array_t* a = hyd_read_array_csv(path, wit_shape(1, n, 0));
    memcpy(out, a->data, (size_t)n * sizeof(int64_t));
    hyd_array_free(a);
}

void wit_read_float_array_csv(const char* path, int64_t n, double* out) {
    hyd_array_t* a = hyd_read_float_array_csv(path, wit_shape(1, n, 0));
    memcpy(out, a->data, (size_t)n * sizeof(double));
    hyd_array_free(a);
}

int64_t wit_write_array_csv(const int64_t* data, int ndims, int64_t d0, int64_t d1, const char* path) {
    hyd_tuple_t s = wit_shape(ndims, d0, d1);
    hyd_array_t* a = hyd_array_alloc(s);
    memcpy(a->data, data, (size_t)hyd_shape_size(s) * sizeof(int64_t));
    int64_t r = hyd_write_array_csv(a, path);
    hyd_array_free(a);
    return r;
}

int64_t wit_write_array_csv_float(const double* data, int ndims, int64_t d0, int64_t d1, const char* path) {
    hyd_tuple_t s = wit_shape(ndims, d0, d1);
    hyd_array_t* a = hyd_array_alloc(s);
    memcpy(a->data, data, (size_t)hyd_shape_size(s) * sizeof(double));
    int64_t r = hyd_write_array_csv_float(a, path);
    hyd_array_free(a);
    return r;
}
