// export.cu -- the embedding boundary on host memory and `hyd_array_t`.
//
// The reference exports a compiled program as `RET hyd_export_<name>(PARAMS)`
// with an extern "C" header that includes hydrangea_runtime.h
// (CodegenC.hs:372-460); host applications link it and free returned arrays
// with hyd_array_free (runtime/hydrangea_runtime.h:333-343).  The functions
// here are what `--backend cuda` export mode provides for the benchmark
// programs: host arrays in, host arrays/scalars out, with the host<->device
// traffic pipelined against the kernels (two streams, double-buffered
// staging: the copy of chunk k+1 overlaps the kernel on chunk k).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "hyd_common.cuh"

namespace hyd {

constexpr int64_t kChunkBytes = 64LL << 20;  // staging chunk per stream

static int stage_pair(Device* d, const char* key, size_t chunk_bytes, unsigned char* stage[2]) {
    void* p = nullptr;
    HYD_TRY(device_buffer(d, key, 2 * chunk_bytes, &p));
    stage[0] = static_cast<unsigned char*>(p);
    stage[1] = stage[0] + chunk_bytes;
    return HYD_CUDA_OK;
}

// Host allocation compatible with the reference's hyd_array_free(): header,
// storage record and zeroed data block each from malloc/calloc, refcount 1.
static hyd_array_t* host_array_alloc(const hyd_tuple_t& shape, size_t elem_size) {
    int64_t size = 1;
    for (int i = 0; i < shape.ndims; ++i) size *= shape.elems[i];
    hyd_array_storage_t* st = (hyd_array_storage_t*)malloc(sizeof(hyd_array_storage_t));
    hyd_array_t* a = (hyd_array_t*)malloc(sizeof(hyd_array_t));
    unsigned char* data = (unsigned char*)calloc((size_t)(size > 0 ? size : 1), elem_size);
    if (!st || !a || !data) {
        free(st);
        free(a);
        free(data);
        return nullptr;
    }
    st->data = data;
    st->refcount = 1;
    a->storage = st;
    a->data = data;
    a->elem_size = elem_size;
    a->shape = shape;
    return a;
}

static int64_t shape_size(const hyd_tuple_t& s) {
    int64_t n = 1;
    for (int i = 0; i < s.ndims; ++i) n *= s.elems[i];
    return n;
}

// resident.cu: the device copy of an attached array (nullptr if not attached)
int resident_device_data(const hyd_array_t* a, const void** out);

[[noreturn]] static void export_fail(const char* what, int status) {
    // Keeps the reference runtime's failure behaviour for exported symbols:
    // message on stderr, exit(1) (runtime/hydrangea_runtime.h:322-328).
    fprintf(stderr, "hydrangea(cuda): %s failed: %s (%s)\n", what, hyd_cuda_status_string(status),
            last_error());
    exit(1);
}

}  // namespace hyd

using namespace hyd;

extern "C" {

int hyd_cuda_weighted_histogram_host(const int64_t* data, int64_t n, int64_t bins, int64_t* hist,
                                     int strategy) {
    HYD_CHECK_ARG(n >= 0 && bins > 0, "weighted_histogram_host: bad sizes");
    HYD_CHECK_ARG(hist != nullptr && (n == 0 || data != nullptr), "weighted_histogram_host: null pointer");
    Device* d = nullptr;
    HYD_TRY(device(&d));
    cudaStream_t s[2];
    HYD_TRY(side_streams(d, s));
    unsigned char* stage[2];
    const int64_t chunk = kChunkBytes / 8;
    HYD_TRY(stage_pair(d, "whist_stage", (size_t)kChunkBytes, stage));
    void* dh = nullptr;
    HYD_TRY(device_buffer(d, "whist_bins", (size_t)bins * 8, &dh));
    HYD_CUDA_TRY(cudaMemsetAsync(dh, 0, (size_t)bins * 8, s[0]));
    cudaEvent_t zeroed;
    HYD_CUDA_TRY(cudaEventCreateWithFlags(&zeroed, cudaEventDisableTiming));
    HYD_CUDA_TRY(cudaEventRecord(zeroed, s[0]));
    HYD_CUDA_TRY(cudaStreamWaitEvent(s[1], zeroed, 0));
    int64_t k = 0;
    for (int64_t off = 0; off < n; off += chunk, ++k) {
        int64_t len = n - off < chunk ? n - off : chunk;
        cudaStream_t st = s[k & 1];
        int64_t* buf = reinterpret_cast<int64_t*>(stage[k & 1]);
        HYD_CUDA_TRY(cudaMemcpyAsync(buf, data + off, (size_t)len * 8, cudaMemcpyHostToDevice, st));
        HYD_TRY(hyd_cuda_weighted_histogram_i64(buf, len, bins, (int64_t*)dh, strategy, st));
    }
    HYD_CUDA_TRY(cudaEventRecord(zeroed, s[1]));
    HYD_CUDA_TRY(cudaStreamWaitEvent(s[0], zeroed, 0));
    HYD_CUDA_TRY(cudaMemcpyAsync(hist, dh, (size_t)bins * 8, cudaMemcpyDeviceToHost, s[0]));
    HYD_CUDA_TRY(cudaStreamSynchronize(s[0]));
    cudaEventDestroy(zeroed);
    return hyd_cuda_check(s[0]);
}

int hyd_cuda_dot_f64_host(const double* xs, const double* ys, int64_t n, double* out) {
    HYD_CHECK_ARG(n >= 0 && out != nullptr, "dot_f64_host: bad arguments");
    HYD_CHECK_ARG(n == 0 || (xs != nullptr && ys != nullptr), "dot_f64_host: null input");
    Device* d = nullptr;
    HYD_TRY(device(&d));
    cudaStream_t s[2];
    HYD_TRY(side_streams(d, s));
    unsigned char* sx[2];
    unsigned char* sy[2];
    const int64_t chunk = kChunkBytes / 8;
    HYD_TRY(stage_pair(d, "dot_stage_x", (size_t)kChunkBytes, sx));
    HYD_TRY(stage_pair(d, "dot_stage_y", (size_t)kChunkBytes, sy));
    const int64_t nchunks = n == 0 ? 1 : (n + chunk - 1) / chunk;
    void* dparts = nullptr;
    HYD_TRY(device_buffer(d, "dot_chunk_parts", (size_t)nchunks * 8, &dparts));
    double* parts = static_cast<double*>(dparts);
    if (n == 0) {
        *out = 0.0;
        return HYD_CUDA_OK;
    }
    for (int64_t k = 0; k < nchunks; ++k) {
        int64_t off = k * chunk;
        int64_t len = n - off < chunk ? n - off : chunk;
        cudaStream_t st = s[k & 1];
        double* bx = reinterpret_cast<double*>(sx[k & 1]);
        double* by = reinterpret_cast<double*>(sy[k & 1]);
        HYD_CUDA_TRY(cudaMemcpyAsync(bx, xs + off, (size_t)len * 8, cudaMemcpyHostToDevice, st));
        HYD_CUDA_TRY(cudaMemcpyAsync(by, ys + off, (size_t)len * 8, cudaMemcpyHostToDevice, st));
        HYD_TRY(hyd_cuda_dot_f64(bx, by, len, parts + k, st));
    }
    HYD_CUDA_TRY(cudaStreamSynchronize(s[0]));
    HYD_CUDA_TRY(cudaStreamSynchronize(s[1]));
    // chunk partials combined in chunk order (deterministic)
    double* hp = (double*)malloc((size_t)nchunks * 8);
    if (!hp) return set_error(HYD_CUDA_ERR_NOMEM, "dot_f64_host: host allocation failed");
    cudaError_t e = cudaMemcpy(hp, parts, (size_t)nchunks * 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        free(hp);
        return set_error(HYD_CUDA_ERR_CUDA, "dot_f64_host: readback failed: %s", cudaGetErrorString(e));
    }
    double acc = 0.0;
    for (int64_t k = 0; k < nchunks; ++k) acc += hp[k];
    free(hp);
    *out = acc;
    return HYD_CUDA_OK;
}

hyd_array_t* hyd_cuda_array_alloc(hyd_tuple_t shape, size_t elem_size) {
    return host_array_alloc(shape, elem_size);
}

// examples/weighted_histogram.hyd with `data` a parameter:
//   scatter (+) (fill [bins] 0) (map (x % bins) data) (map (x * x) data)
hyd_array_t* hyd_export_weighted_histogram(hyd_array_t* data, int64_t bins) {
    if (!data || data->shape.ndims != 1 || data->elem_size != 8 || bins <= 0) {
        set_error(HYD_CUDA_ERR_INVALID, "expected a 1-D int64 array and bins > 0");
        export_fail("hyd_export_weighted_histogram", HYD_CUDA_ERR_INVALID);
    }
    hyd_tuple_t shape;
    memset(&shape, 0, sizeof shape);
    shape.ndims = 1;
    shape.elems[0] = bins;
    hyd_array_t* out = host_array_alloc(shape, 8);
    if (!out) export_fail("hyd_export_weighted_histogram", HYD_CUDA_ERR_NOMEM);
    const int64_t n = shape_size(data->shape);
    const void* ddata = nullptr;
    int s = resident_device_data(data, &ddata);
    if (s == HYD_CUDA_OK && ddata) {
        // an attached array: its device copy, no host->device traffic
        Device* d = nullptr;
        cudaStream_t st[2];
        void* dh = nullptr;
        s = device(&d);
        if (s == HYD_CUDA_OK) s = side_streams(d, st);
        if (s == HYD_CUDA_OK) s = device_buffer(d, "whist_bins", (size_t)bins * 8, &dh);
        if (s == HYD_CUDA_OK && cudaMemsetAsync(dh, 0, (size_t)bins * 8, st[0]) != cudaSuccess)
            s = set_error(HYD_CUDA_ERR_CUDA, "weighted_histogram: clearing the bins failed");
        if (s == HYD_CUDA_OK)
            s = hyd_cuda_weighted_histogram_i64((const int64_t*)ddata, n, bins, (int64_t*)dh, HYD_SCATTER_AUTO, st[0]);
        if (s == HYD_CUDA_OK && cudaMemcpyAsync(out->data, dh, (size_t)bins * 8, cudaMemcpyDeviceToHost, st[0]) !=
                                    cudaSuccess)
            s = set_error(HYD_CUDA_ERR_CUDA, "weighted_histogram: reading the bins back failed");
        if (s == HYD_CUDA_OK && cudaStreamSynchronize(st[0]) != cudaSuccess)
            s = set_error(HYD_CUDA_ERR_CUDA, "weighted_histogram: synchronize failed");
        if (s == HYD_CUDA_OK) s = hyd_cuda_check(st[0]);
    } else if (s == HYD_CUDA_OK) {
        s = hyd_cuda_weighted_histogram_host((const int64_t*)data->data, n, bins, (int64_t*)out->data,
                                             HYD_SCATTER_AUTO);
    }
    if (s != HYD_CUDA_OK) export_fail("hyd_export_weighted_histogram", s);
    return out;
}

// examples/dot.hyd shape with parameters: reduce (+) 0.0 (zipwith (*) xs ys)
double hyd_export_dot(hyd_array_t* xs, hyd_array_t* ys) {
    if (!xs || !ys || xs->elem_size != 8 || ys->elem_size != 8 ||
        shape_size(xs->shape) != shape_size(ys->shape)) {
        set_error(HYD_CUDA_ERR_INVALID, "expected two float64 arrays of equal size");
        export_fail("hyd_export_dot", HYD_CUDA_ERR_INVALID);
    }
    double r = 0.0;
    const int64_t n = shape_size(xs->shape);
    const void* dx = nullptr;
    const void* dy = nullptr;
    int s = resident_device_data(xs, &dx);
    if (s == HYD_CUDA_OK) s = resident_device_data(ys, &dy);
    if (s == HYD_CUDA_OK && dx && dy) {
        // both arrays attached: their device copies, no host->device traffic
        Device* d = nullptr;
        cudaStream_t st[2];
        void* dout = nullptr;
        s = device(&d);
        if (s == HYD_CUDA_OK) s = side_streams(d, st);
        if (s == HYD_CUDA_OK) s = device_buffer(d, "export_dot_out", 8, &dout);
        if (s == HYD_CUDA_OK) s = hyd_cuda_dot_f64((const double*)dx, (const double*)dy, n, (double*)dout, st[0]);
        if (s == HYD_CUDA_OK && cudaMemcpyAsync(&r, dout, 8, cudaMemcpyDeviceToHost, st[0]) != cudaSuccess)
            s = set_error(HYD_CUDA_ERR_CUDA, "dot: reading the result back failed");
        if (s == HYD_CUDA_OK && cudaStreamSynchronize(st[0]) != cudaSuccess)
            s = set_error(HYD_CUDA_ERR_CUDA, "dot: synchronize failed");
        if (s == HYD_CUDA_OK) s = hyd_cuda_check(st[0]);
    } else if (s == HYD_CUDA_OK) {
        s = hyd_cuda_dot_f64_host((const double*)xs->data, (const double*)ys->data, n, &r);
    }
    if (s != HYD_CUDA_OK) export_fail("hyd_export_dot", s);
    return r;
}

}  // extern "C"
