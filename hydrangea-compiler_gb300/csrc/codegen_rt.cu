// codegen_rt.cu -- the host-side runtime calls that code generated for
// `--backend cuda` makes around the device primitives.
//
// The reference C backend's generated code calls helpers of
// runtime/hydrangea_runtime.h: array allocation and release (:292-343),
// hyd_get_env_int (:602-616), the printers main uses for every zero-argument
// procedure (hyd_print_int/_double/_array/_float_array, :460-536), and exits
// with a message on any failure (:322-328).  Generated CUDA host code needs the
// same services plus device buffers and the copies between them and the
// hyd_array_t host arrays that procedures return.  These entry points provide
// them with the reference's behaviour: output bytes identical to the printers
// above, and a message on stderr followed by exit(1) instead of a status, so
// the emitted code carries no error handling of its own.  All device work is
// ordered on the legacy default stream, like the C backend's single thread of
// control between loop nests.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "hyd_common.cuh"

using namespace hyd;

extern "C" {

void hyd_cuda_gen_check(int status, const char* what) {
    if (status == HYD_CUDA_OK) return;
    fprintf(stderr, "hydrangea(cuda): %s failed: %s (%s)\n", what ? what : "runtime call",
            hyd_cuda_status_string(status), last_error());
    exit(1);
}

void* hyd_cuda_gen_alloc(int64_t bytes) {
    if (bytes < 0) {
        set_error(HYD_CUDA_ERR_INVALID, "negative size %lld", (long long)bytes);
        hyd_cuda_gen_check(HYD_CUDA_ERR_INVALID, "device allocation");
    }
    hyd_cuda_gen_check(hyd_cuda_init(), "hyd_cuda_init");
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, (size_t)(bytes > 0 ? bytes : 1));
    if (e != cudaSuccess) {
        set_error(HYD_CUDA_ERR_NOMEM, "cudaMalloc of %lld bytes: %s", (long long)bytes, cudaGetErrorString(e));
        hyd_cuda_gen_check(HYD_CUDA_ERR_NOMEM, "device allocation");
    }
    return p;
}

void hyd_cuda_gen_free(void* d) {
    if (d) cudaFree(d);
}

void hyd_cuda_gen_zero(void* d, int64_t bytes) {
    if (bytes <= 0) return;
    const cudaError_t e = cudaMemsetAsync(d, 0, (size_t)bytes, 0);
    if (e != cudaSuccess) {
        set_error(HYD_CUDA_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
        hyd_cuda_gen_check(HYD_CUDA_ERR_CUDA, "device fill");
    }
}

static int64_t shape_elems(const hyd_tuple_t& s) {
    int64_t n = 1;
    for (int i = 0; i < s.ndims; ++i) n *= s.elems[i];
    return n;
}

// A device copy of a host array's data (the caller frees it with hyd_cuda_gen_free).
void* hyd_cuda_gen_upload(const hyd_array_t* a) {
    if (!a) {
        set_error(HYD_CUDA_ERR_INVALID, "null array");
        hyd_cuda_gen_check(HYD_CUDA_ERR_INVALID, "upload");
    }
    const int64_t bytes = shape_elems(a->shape) * (int64_t)a->elem_size;
    void* d = hyd_cuda_gen_alloc(bytes);
    if (bytes > 0) {
        const cudaError_t e = cudaMemcpy(d, a->data, (size_t)bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            set_error(HYD_CUDA_ERR_CUDA, "cudaMemcpy: %s", cudaGetErrorString(e));
            hyd_cuda_gen_check(HYD_CUDA_ERR_CUDA, "upload");
        }
    }
    return d;
}

// A new host array (reference allocator layout, refcount 1) holding the device
// buffer's first shape-size elements; device errors raised by the kernels that
// produced it are reported here.
hyd_array_t* hyd_cuda_gen_download(const void* d, hyd_tuple_t shape, size_t elem_size) {
    hyd_cuda_gen_check(hyd_cuda_check(nullptr), "device computation");
    hyd_array_t* a = hyd_cuda_array_alloc(shape, elem_size);
    if (!a) {
        set_error(HYD_CUDA_ERR_NOMEM, "host array allocation");
        hyd_cuda_gen_check(HYD_CUDA_ERR_NOMEM, "download");
    }
    const int64_t bytes = shape_elems(shape) * (int64_t)elem_size;
    if (bytes > 0) {
        const cudaError_t e = cudaMemcpy(a->data, d, (size_t)bytes, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            set_error(HYD_CUDA_ERR_CUDA, "cudaMemcpy: %s", cudaGetErrorString(e));
            hyd_cuda_gen_check(HYD_CUDA_ERR_CUDA, "download");
        }
    }
    return a;
}

int64_t hyd_cuda_gen_read_i64(const int64_t* d) {
    hyd_cuda_gen_check(hyd_cuda_check(nullptr), "device computation");
    int64_t v = 0;
    if (cudaMemcpy(&v, d, sizeof v, cudaMemcpyDeviceToHost) != cudaSuccess) {
        set_error(HYD_CUDA_ERR_CUDA, "cudaMemcpy of a scalar");
        hyd_cuda_gen_check(HYD_CUDA_ERR_CUDA, "read back");
    }
    return v;
}

double hyd_cuda_gen_read_f64(const double* d) {
    hyd_cuda_gen_check(hyd_cuda_check(nullptr), "device computation");
    double v = 0.0;
    if (cudaMemcpy(&v, d, sizeof v, cudaMemcpyDeviceToHost) != cudaSuccess) {
        set_error(HYD_CUDA_ERR_CUDA, "cudaMemcpy of a scalar");
        hyd_cuda_gen_check(HYD_CUDA_ERR_CUDA, "read back");
    }
    return v;
}

// The reference runtime's hyd_array_free: drop one reference to the storage,
// free data and storage at zero, then the header.
void hyd_cuda_gen_array_free(hyd_array_t* a) {
    if (!a) return;
    if (a->storage && --a->storage->refcount == 0) {
        free(a->storage->data);
        free(a->storage);
    }
    free(a);
}

// get_env_int: the value of an environment variable as a base-10 integer; a
// missing or malformed value is a message and exit(1).
int64_t hyd_cuda_gen_get_env_int(const char* name) {
    const char* val = getenv(name);
    if (!val) {
        fprintf(stderr, "get_env_int: environment variable '%s' not set\n", name);
        exit(1);
    }
    char* end = nullptr;
    const long long r = strtoll(val, &end, 10);
    if (*end != '\0' || end == val) {
        fprintf(stderr, "get_env_int: environment variable '%s' is not an integer: '%s'\n", name, val);
        exit(1);
    }
    return (int64_t)r;
}

// ---- printers: the reference's output format --------------------------------
void hyd_cuda_gen_print_int(int64_t v) { printf("%lld\n", (long long)v); }

void hyd_cuda_gen_print_double(double v) { printf("%.17g\n", v); }

static void print_shape(const hyd_tuple_t& s) {
    printf("] (shape: [");
    for (int i = 0; i < s.ndims; ++i) {
        if (i > 0) printf(", ");
        printf("%lld", (long long)s.elems[i]);
    }
    printf("])\n");
}

void hyd_cuda_gen_print_array(const hyd_array_t* a) {
    const int64_t n = shape_elems(a->shape);
    printf("[");
    for (int64_t i = 0; i < n; ++i) {
        int64_t v;
        memcpy(&v, a->data + (size_t)i * a->elem_size, sizeof v);
        if (i > 0) printf(", ");
        printf("%lld", (long long)v);
    }
    print_shape(a->shape);
}

void hyd_cuda_gen_print_float_array(const hyd_array_t* a) {
    const int64_t n = shape_elems(a->shape);
    printf("[");
    for (int64_t i = 0; i < n; ++i) {
        double v;
        memcpy(&v, a->data + (size_t)i * a->elem_size, sizeof v);
        if (i > 0) printf(", ");
        printf("%.17g", v);
    }
    print_shape(a->shape);
}

}  // extern "C"
