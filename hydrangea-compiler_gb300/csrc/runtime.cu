// runtime.cu -- lifecycle, error reporting, per-device context, per-stream
// workspaces and the seeded input generators.
//
// The reference runtime reports failures by printing and calling exit(1)
// (runtime/hydrangea_runtime.h:322-328); this runtime returns status codes and
// keeps a thread-local message instead, so an embedding host decides.
#include <cstdlib>
#include <cstring>
#include <vector>

#include "hyd_common.cuh"

namespace hyd {
void release_map_kernels();      // jit_map.cu
void release_resident_arrays();  // resident.cu
void release_export_memos();     // stencil_more.cu
}

namespace hyd {

static thread_local char g_last_error[1024] = "";

int set_error(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
    return status;
}

const char* last_error() { return g_last_error; }

static std::mutex g_devices_mu;
static std::vector<Device*> g_devices;  // indexed by device id

int device(Device** out) {
    int dev = 0;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return set_error(HYD_CUDA_ERR_NO_DEVICE, "no CUDA device available (%s)",
                         e == cudaSuccess ? "device count 0" : cudaGetErrorString(e));
    }
    HYD_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_devices_mu);
    if ((int)g_devices.size() <= dev) g_devices.resize(dev + 1, nullptr);
    if (g_devices[dev] == nullptr) {
        Device* d = new Device();
        d->id = dev;
        cudaError_t e1 = cudaDeviceGetAttribute(&d->sm_count, cudaDevAttrMultiProcessorCount, dev);
        cudaError_t e2 =
            cudaDeviceGetAttribute(&d->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaError_t e3 = cudaMalloc(&d->d_err, sizeof(unsigned));
        cudaError_t e4 = e3 == cudaSuccess ? cudaMemset(d->d_err, 0, sizeof(unsigned)) : e3;
        if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess || e4 != cudaSuccess) {
            if (e3 == cudaSuccess) cudaFree(d->d_err);
            delete d;
            return set_error(HYD_CUDA_ERR_CUDA, "device %d context set-up failed", dev);
        }
        g_devices[dev] = d;
    }
    *out = g_devices[dev];
    return HYD_CUDA_OK;
}

int workspace(cudaStream_t stream, size_t bytes, unsigned** counters, void** scratch) {
    Device* d = nullptr;
    HYD_TRY(device(&d));
    std::lock_guard<std::mutex> lock(d->mu);
    Workspace& w = d->ws[stream];
    size_t need = kCounterBytes + ((bytes + 255) & ~(size_t)255);
    if (w.bytes < need) {
        if (w.base) {
            HYD_CUDA_TRY(cudaStreamSynchronize(stream));
            HYD_CUDA_TRY(cudaFree(w.base));
            w.base = nullptr;
            w.bytes = 0;
        }
        size_t cap = need < ((size_t)1 << 20) ? ((size_t)1 << 20) : need + need / 4;
        void* p = nullptr;
        HYD_CUDA_TRY(cudaMalloc(&p, cap));
        HYD_CUDA_TRY(cudaMemsetAsync(p, 0, kCounterBytes, stream));
        w.base = static_cast<unsigned char*>(p);
        w.bytes = cap;
    }
    if (counters) *counters = reinterpret_cast<unsigned*>(w.base);
    if (scratch) *scratch = w.base + kCounterBytes;
    return HYD_CUDA_OK;
}

int device_buffer(Device* d, const char* key, size_t bytes, void** p) {
    std::lock_guard<std::mutex> lock(d->mu);
    Workspace& w = d->bufs[key];
    if (w.bytes < bytes) {
        if (w.base) {
            HYD_CUDA_TRY(cudaDeviceSynchronize());
            HYD_CUDA_TRY(cudaFree(w.base));
            w.base = nullptr;
            w.bytes = 0;
        }
        void* q = nullptr;
        HYD_CUDA_TRY(cudaMalloc(&q, bytes));
        w.base = static_cast<unsigned char*>(q);
        w.bytes = bytes;
    }
    *p = w.base;
    return HYD_CUDA_OK;
}

int side_streams(Device* d, cudaStream_t out[2]) {
    std::lock_guard<std::mutex> lock(d->mu);
    for (int i = 0; i < 2; ++i) {
        if (!d->side[i]) HYD_CUDA_TRY(cudaStreamCreateWithFlags(&d->side[i], cudaStreamNonBlocking));
        out[i] = d->side[i];
    }
    return HYD_CUDA_OK;
}

int configure_kernel(const void* fn, const Device* d, bool nonportable_cluster) {
    static std::mutex mu;
    static std::unordered_map<const void*, unsigned> done;  // kernel -> device bit mask
    std::lock_guard<std::mutex> lock(mu);
    unsigned& mask = done[fn];
    const unsigned bit = 1u << (d->id & 31);
    if (mask & bit) return HYD_CUDA_OK;
    // dynamic + static shared memory may not exceed the opt-in maximum
    cudaFuncAttributes fa;
    HYD_CUDA_TRY(cudaFuncGetAttributes(&fa, fn));
    HYD_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      d->max_smem_optin - (int)fa.sharedSizeBytes));
    if (nonportable_cluster)
        HYD_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    mask |= bit;
    return HYD_CUDA_OK;
}

// ------------------------------------------------------------ generators ----
__global__ void fill_uniform_f64_kernel(double* out, int64_t n, uint64_t seed_mixed, double lo,
                                        double scale) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double u = (double)(rand_u64(seed_mixed, (uint64_t)i) >> 11) * 0x1.0p-53;
        // round(lo + round(scale*u)), exactly as the oracle's unfused C
        out[i] = __dadd_rn(lo, __dmul_rn(scale, u));
    }
}

__global__ void fill_uniform_i64_kernel(int64_t* out, int64_t n, uint64_t seed_mixed,
                                        uint64_t bound) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = (int64_t)(rand_u64(seed_mixed, (uint64_t)i) % bound);
}

static int grid_for(int64_t n, int threads) {
    Device* d = nullptr;
    if (device(&d) != HYD_CUDA_OK) return 1;
    int64_t want = (n + threads - 1) / threads;
    int64_t cap = (int64_t)d->sm_count * 8;
    return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

}  // namespace hyd

using namespace hyd;

extern "C" {

int hyd_cuda_version(void) { return 100; }

const char* hyd_cuda_last_error(void) { return last_error(); }

const char* hyd_cuda_status_string(int status) {
    switch (status) {
        case HYD_CUDA_OK: return "ok";
        case HYD_CUDA_ERR_INVALID: return "invalid argument";
        case HYD_CUDA_ERR_NOMEM: return "out of memory";
        case HYD_CUDA_ERR_CUDA: return "CUDA error";
        case HYD_CUDA_ERR_NO_DEVICE: return "no CUDA device";
        case HYD_CUDA_ERR_BOUNDS: return "index out of bounds";
        case HYD_CUDA_ERR_TIMEOUT: return "device wait timed out";
        case HYD_CUDA_ERR_BUDGET: return "HBM budget exceeded";
        case HYD_CUDA_ERR_CANCELLED: return "cancelled";
        case HYD_CUDA_ERR_UNSUPPORTED: return "unsupported";
        default: return "unknown status";
    }
}

int hyd_cuda_init(void) {
    Device* d = nullptr;
    return device(&d);
}

extern "C" void hyd_cuda_stencil_release_graphs(void);

void hyd_cuda_cleanup(void) {
    hyd_cuda_stencil_release_graphs();
    release_map_kernels();
    release_resident_arrays();
    release_export_memos();
    std::lock_guard<std::mutex> lock(g_devices_mu);
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) cur = 0;
    for (Device* d : g_devices) {
        if (!d) continue;
        cudaSetDevice(d->id);
        cudaDeviceSynchronize();
        for (auto& kv : d->ws)
            if (kv.second.base) cudaFree(kv.second.base);
        for (auto& kv : d->bufs)
            if (kv.second.base) cudaFree(kv.second.base);
        for (cudaStream_t s : d->side)
            if (s) cudaStreamDestroy(s);
        if (d->d_err) cudaFree(d->d_err);
        delete d;
    }
    g_devices.clear();
    cudaSetDevice(cur);
    cudaGetLastError();
}

int hyd_cuda_device_sm_count(void) {
    Device* d = nullptr;
    int s = device(&d);
    return s == HYD_CUDA_OK ? d->sm_count : -s;
}

int hyd_cuda_check(void* stream) {
    Device* d = nullptr;
    HYD_TRY(device(&d));
    HYD_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
    unsigned err = 0;
    HYD_CUDA_TRY(cudaMemcpy(&err, d->d_err, sizeof err, cudaMemcpyDeviceToHost));
    if (err) {
        HYD_CUDA_TRY(cudaMemset(d->d_err, 0, sizeof(unsigned)));
        if (err & ERRBIT_BOUNDS)
            return set_error(HYD_CUDA_ERR_BOUNDS, "a kernel saw an index outside its destination");
        return set_error(HYD_CUDA_ERR_TIMEOUT, "a bounded device wait gave up (error word 0x%x)", err);
    }
    return HYD_CUDA_OK;
}

int hyd_cuda_fill_uniform_f64(double* out, int64_t n, uint64_t seed, double lo, double hi,
                              void* stream) {
    HYD_CHECK_ARG(n >= 0, "fill_uniform_f64: negative length %lld", (long long)n);
    HYD_CHECK_ARG(n == 0 || out != nullptr, "fill_uniform_f64: null output");
    if (n == 0) return HYD_CUDA_OK;
    fill_uniform_f64_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(out, n, mix64(seed),
                                                                             lo, hi - lo);
    return launch_check("fill_uniform_f64");
}

int hyd_cuda_fill_uniform_i64(int64_t* out, int64_t n, uint64_t seed, int64_t bound,
                              void* stream) {
    HYD_CHECK_ARG(n >= 0, "fill_uniform_i64: negative length %lld", (long long)n);
    HYD_CHECK_ARG(bound > 0, "fill_uniform_i64: bound must be positive");
    HYD_CHECK_ARG(n == 0 || out != nullptr, "fill_uniform_i64: null output");
    if (n == 0) return HYD_CUDA_OK;
    fill_uniform_i64_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
        out, n, mix64(seed), (uint64_t)bound);
    return launch_check("fill_uniform_i64");
}

}  // extern "C"
