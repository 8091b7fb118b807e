// resident.cu -- device-resident copies of host arrays for the export path.
//
// The reference keeps every array in host memory (hyd_array_t over refcounted
// storage, runtime/hydrangea_runtime.h:220-235, :292-343).  Its Metal export
// lifecycle uploads the zero-argument array bindings once, at init, and keeps
// them as persistent GPU buffers across dispatches (CodegenMSL.hs:1253-1300).
// Here an embedding host can make any host array device-resident:
//   * hyd_cuda_array_attach uploads it once and keeps a device copy beside
//     storage->data, with a validity flag;
//   * the hyd_export_* entry points read attached arrays from that copy
//     instead of streaming the host data to the device on every call;
//   * the host declares its own writes with hyd_cuda_array_host_modified (the
//     next use uploads again; the reference runtime has no hook that would
//     see them) and calls hyd_cuda_array_detach before hyd_array_free.
// A copy is keyed by (storage record, data pointer, byte size): a view with a
// different extent is a different entry, and an address reused after a free
// without a detach never matches a stale copy of another size.
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "hyd_common.cuh"

namespace hyd {

struct ResidentKey {
    const void* storage;
    const void* data;
    size_t bytes;
    bool operator<(const ResidentKey& o) const {
        return std::tie(storage, data, bytes) < std::tie(o.storage, o.data, o.bytes);
    }
};

struct ResidentCopy {
    void* dev = nullptr;
    int device = -1;
    bool valid = false;  // the device copy equals the host data
};

static std::mutex g_res_mu;
static std::map<ResidentKey, ResidentCopy> g_res;
static int64_t g_res_uploads = 0;

static int64_t array_bytes(const hyd_array_t* a) {
    int64_t n = 1;
    for (int i = 0; i < a->shape.ndims; ++i) n *= a->shape.elems[i];
    return n * (int64_t)a->elem_size;
}

static int check_array(const hyd_array_t* a, const char* what) {
    if (!a || !a->storage || (!a->data && array_bytes(a) > 0) || a->shape.ndims < 0 || a->shape.ndims > 8)
        return set_error(HYD_CUDA_ERR_INVALID, "%s: not a valid array", what);
    if (array_bytes(a) < 0) return set_error(HYD_CUDA_ERR_INVALID, "%s: negative extent", what);
    return HYD_CUDA_OK;
}

static ResidentKey key_of(const hyd_array_t* a) {
    return ResidentKey{a->storage, a->data, (size_t)array_bytes(a)};
}

// Uploads the host data of `a` into its copy if the copy is stale (caller
// holds g_res_mu).
static int refresh(const hyd_array_t* a, ResidentCopy& c) {
    if (c.valid) return HYD_CUDA_OK;
    const size_t bytes = (size_t)array_bytes(a);
    if (bytes) HYD_CUDA_TRY(cudaMemcpy(c.dev, a->data, bytes, cudaMemcpyHostToDevice));
    c.valid = true;
    ++g_res_uploads;
    return HYD_CUDA_OK;
}

int resident_device_data(const hyd_array_t* a, const void** out) {
    *out = nullptr;
    if (!a) return HYD_CUDA_OK;
    std::lock_guard<std::mutex> lock(g_res_mu);
    auto it = g_res.find(key_of(a));
    if (it == g_res.end()) return HYD_CUDA_OK;
    int cur = 0;
    HYD_CUDA_TRY(cudaGetDevice(&cur));
    if (it->second.device != cur) return HYD_CUDA_OK;  // resident on another device: not usable here
    HYD_TRY(refresh(a, it->second));
    *out = it->second.dev;
    return HYD_CUDA_OK;
}

void release_resident_arrays() {
    std::lock_guard<std::mutex> lock(g_res_mu);
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) cur = 0;
    for (auto& kv : g_res) {
        if (!kv.second.dev) continue;
        cudaSetDevice(kv.second.device);
        cudaFree(kv.second.dev);
    }
    g_res.clear();
    cudaSetDevice(cur);
    cudaGetLastError();
}

}  // namespace hyd

using namespace hyd;

extern "C" {

int hyd_cuda_array_attach(hyd_array_t* a) {
    HYD_TRY(check_array(a, "array_attach"));
    Device* d = nullptr;
    HYD_TRY(device(&d));
    std::lock_guard<std::mutex> lock(g_res_mu);
    const ResidentKey k = key_of(a);
    auto it = g_res.find(k);
    if (it == g_res.end()) {
        ResidentCopy c;
        c.device = d->id;
        const size_t bytes = k.bytes ? k.bytes : 1;
        HYD_CUDA_TRY(cudaMalloc(&c.dev, bytes));
        it = g_res.emplace(k, c).first;
    }
    return refresh(a, it->second);
}

int hyd_cuda_array_host_modified(hyd_array_t* a) {
    HYD_TRY(check_array(a, "array_host_modified"));
    std::lock_guard<std::mutex> lock(g_res_mu);
    auto it = g_res.find(key_of(a));
    if (it == g_res.end()) return set_error(HYD_CUDA_ERR_INVALID, "array_host_modified: array is not attached");
    it->second.valid = false;
    return HYD_CUDA_OK;
}

int hyd_cuda_array_detach(hyd_array_t* a) {
    HYD_TRY(check_array(a, "array_detach"));
    std::lock_guard<std::mutex> lock(g_res_mu);
    auto it = g_res.find(key_of(a));
    if (it == g_res.end()) return set_error(HYD_CUDA_ERR_INVALID, "array_detach: array is not attached");
    int cur = 0;
    HYD_CUDA_TRY(cudaGetDevice(&cur));
    if (it->second.device != cur) HYD_CUDA_TRY(cudaSetDevice(it->second.device));
    const cudaError_t e = cudaFree(it->second.dev);
    if (it->second.device != cur) cudaSetDevice(cur);
    g_res.erase(it);
    HYD_CUDA_TRY(e);
    return HYD_CUDA_OK;
}

const void* hyd_cuda_array_device_data(hyd_array_t* a) {
    const void* p = nullptr;
    if (check_array(a, "array_device_data") != HYD_CUDA_OK) return nullptr;
    if (resident_device_data(a, &p) != HYD_CUDA_OK) return nullptr;
    return p;
}

int hyd_cuda_array_resident_stats(int64_t* entries, int64_t* uploads, int64_t* bytes) {
    std::lock_guard<std::mutex> lock(g_res_mu);
    int64_t b = 0;
    for (auto& kv : g_res) b += (int64_t)kv.first.bytes;
    if (entries) *entries = (int64_t)g_res.size();
    if (uploads) *uploads = g_res_uploads;
    if (bytes) *bytes = b;
    return HYD_CUDA_OK;
}

}  // extern "C"
