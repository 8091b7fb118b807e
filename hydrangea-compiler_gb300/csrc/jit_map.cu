// jit_map.cu -- fused map / zipwith / generate chains compiled at run time.
//
// The C backend turns a fused chain such as
//   reduce (+) 0.0 (map (fn x => x *. 2.0 +. 1.0) (map (fn x => x -. 0.5)
//     (map (fn x => x *. x) (generate [n] (fn [i] => float_of i /. float_of n)))))
// (bench/map_chain/map_chain.hyd) into one loop whose body evaluates the
// composed element expression (CodegenC.hs:1328-1353 for the reduced form).
// Here the generated element body -- C statements over the inputs' elements
// x0..x7 and the index i that assign `v` -- is compiled once per body and
// device with NVRTC into a kernel that:
//   * walks the elements as a grid-stride loop over pairs, with 128-bit
//     (double2) loads and stores when every pointer is 16-byte aligned;
//   * evaluates the body with IEEE round-to-nearest operations and no
//     contraction (--fmad=false), so each element equals the C backend's;
//   * optionally writes the elements and/or reduces them with (+): per-thread
//     sums, a fixed shuffle tree per block, block partials combined in block
//     order by the last block -- the same bits on every run.
// NVRTC is loaded with dlopen on first use; without it the call reports
// HYD_CUDA_ERR_UNSUPPORTED.
#include <dlfcn.h>
#include <nvrtc.h>

#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "hyd_common.cuh"

namespace hyd {

struct Nvrtc {
    bool tried = false, ok = false;
    decltype(&nvrtcCreateProgram) create = nullptr;
    decltype(&nvrtcCompileProgram) compile = nullptr;
    decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
    decltype(&nvrtcGetProgramLog) log = nullptr;
    decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
    decltype(&nvrtcGetCUBIN) cubin = nullptr;
    decltype(&nvrtcDestroyProgram) destroy = nullptr;
};

static std::mutex g_jit_mu;
static Nvrtc g_nvrtc;

static bool load_nvrtc_locked() {
    if (g_nvrtc.tried) return g_nvrtc.ok;
    g_nvrtc.tried = true;
    std::vector<std::string> names = {"libnvrtc.so.13", "libnvrtc.so"};
    if (const char* home = getenv("CUDA_HOME")) names.push_back(std::string(home) + "/lib64/libnvrtc.so.13");
    names.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");  // the toolkit's default install location
    void* h = nullptr;
    for (const std::string& n : names)
        if ((h = dlopen(n.c_str(), RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
    if (!h) return false;
    g_nvrtc.create = (decltype(&nvrtcCreateProgram))dlsym(h, "nvrtcCreateProgram");
    g_nvrtc.compile = (decltype(&nvrtcCompileProgram))dlsym(h, "nvrtcCompileProgram");
    g_nvrtc.log_size = (decltype(&nvrtcGetProgramLogSize))dlsym(h, "nvrtcGetProgramLogSize");
    g_nvrtc.log = (decltype(&nvrtcGetProgramLog))dlsym(h, "nvrtcGetProgramLog");
    g_nvrtc.cubin_size = (decltype(&nvrtcGetCUBINSize))dlsym(h, "nvrtcGetCUBINSize");
    g_nvrtc.cubin = (decltype(&nvrtcGetCUBIN))dlsym(h, "nvrtcGetCUBIN");
    g_nvrtc.destroy = (decltype(&nvrtcDestroyProgram))dlsym(h, "nvrtcDestroyProgram");
    g_nvrtc.ok = g_nvrtc.create && g_nvrtc.compile && g_nvrtc.log_size && g_nvrtc.log && g_nvrtc.cubin_size &&
                 g_nvrtc.cubin && g_nvrtc.destroy;
    return g_nvrtc.ok;
}

constexpr int kMapMaxInputs = 8;
constexpr int kMapThreads = 256;

// Kernel source for `body` over `nin` inputs of element type T ("double" or
// "long long").  int64 sums wrap (accumulated as unsigned), as the C backend's
// int64 arithmetic does on every target it runs on.
static std::string map_source(const std::string& body, int nin, bool i64) {
    const std::string T = i64 ? "long long" : "double";
    const std::string T2 = i64 ? "longlong2" : "double2";
    const std::string A = i64 ? "unsigned long long" : "double";  // accumulator
    const std::string zero = i64 ? "0LL" : "0.0";
    std::string s;
    s += "__device__ __forceinline__ " + T + " hyd_elem(long long i";
    for (int k = 0; k < kMapMaxInputs; ++k) s += ", " + T + " x" + std::to_string(k);
    s += ") {\n  " + T + " v = " + zero + ";\n  (void)i;\n";
    for (int k = 0; k < kMapMaxInputs; ++k) s += "  (void)x" + std::to_string(k) + ";\n";
    s += "  {\n" + body + "\n  }\n  return v;\n}\n";
    s += "extern \"C\" __global__ void __launch_bounds__(256) hyd_map_kernel(";
    for (int k = 0; k < kMapMaxInputs; ++k) s += "const " + T + "* __restrict__ p" + std::to_string(k) + ", ";
    s += "long long n, " + T + "* __restrict__ out, " + A + "* __restrict__ partials, unsigned int* counter, " + A +
         "* __restrict__ sum, int vec) {\n"
         "  " + A + " acc = 0;\n"
         "  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n"
         "  const long long nt = (long long)gridDim.x * blockDim.x;\n"
         "  if (vec == 2) {\n"
         "    const long long nq = n >> 2;\n"
         "    long long q = t;\n"
         "    for (; q < nq; q += 2 * nt) {\n"
         "      const bool two = q + nt < nq;\n";
    // 32-byte vectors, two per lane per step (8 elements), all loads first
    const std::string LD = i64 ? "ld.global.nc.L1::no_allocate.v4.u64" : "ld.global.nc.L1::no_allocate.v4.f64";
    const std::string ST = i64 ? "st.global.v4.u64" : "st.global.v4.f64";
    const std::string RC = i64 ? "l" : "d";
    for (int k = 0; k < kMapMaxInputs; ++k) {
        const std::string ks = std::to_string(k);
        s += "      " + T + " a" + ks + "[8];\n";
        if (k < nin) {
            for (int h = 0; h < 2; ++h) {
                const std::string hs = std::to_string(h);
                s += std::string("      ") + (h ? "if (two) " : "") + "asm volatile(\"" + LD +
                     " {%0,%1,%2,%3}, [%4];\" : \"=" + RC + "\"(a" + ks + "[" + std::to_string(4 * h) + "]), \"=" + RC +
                     "\"(a" + ks + "[" + std::to_string(4 * h + 1) + "]), \"=" + RC + "\"(a" + ks + "[" +
                     std::to_string(4 * h + 2) + "]), \"=" + RC + "\"(a" + ks + "[" + std::to_string(4 * h + 3) +
                     "]) : \"l\"(p" + ks + " + 4 * (q + " + hs + " * nt)));\n";
                if (h) s += "      else { a" + ks + "[4] = a" + ks + "[5] = a" + ks + "[6] = a" + ks + "[7] = " + zero + "; }\n";
            }
        } else {
            s += "      for (int u = 0; u < 8; ++u) a" + ks + "[u] = " + zero + ";\n";
        }
    }
    s += "      " + T + " w[8];\n"
         "      #pragma unroll\n"
         "      for (int u = 0; u < 8; ++u) w[u] = hyd_elem(4 * (q + (u >> 2) * nt) + (u & 3)";
    for (int k = 0; k < kMapMaxInputs; ++k) s += ", a" + std::to_string(k) + "[u]";
    s += ");\n"
         "      if (out) {\n"
         "        asm volatile(\"" + ST + " [%0], {%1,%2,%3,%4};\" :: \"l\"(out + 4 * q), \"" + RC + "\"(w[0]), \"" +
         RC + "\"(w[1]), \"" + RC + "\"(w[2]), \"" + RC + "\"(w[3]) : \"memory\");\n"
         "        if (two) asm volatile(\"" + ST + " [%0], {%1,%2,%3,%4};\" :: \"l\"(out + 4 * (q + nt)), \"" + RC +
         "\"(w[4]), \"" + RC + "\"(w[5]), \"" + RC + "\"(w[6]), \"" + RC + "\"(w[7]) : \"memory\");\n"
         "      }\n"
         "      #pragma unroll\n"
         "      for (int u = 0; u < 4; ++u) acc += (" + A + ")w[u];\n"
         "      if (two) {\n"
         "        #pragma unroll\n"
         "        for (int u = 4; u < 8; ++u) acc += (" + A + ")w[u];\n"
         "      }\n"
         "    }\n"
         "    for (long long i = 4 * nq + t; i < n; i += nt) {\n"
         "      const " + T + " v = hyd_elem(i";
    for (int k = 0; k < kMapMaxInputs; ++k) s += k < nin ? ", p" + std::to_string(k) + "[i]" : ", " + zero;
    s += ");\n"
         "      if (out) out[i] = v;\n"
         "      acc += (" + A + ")v;\n"
         "    }\n"
         "  } else if (vec) {\n"
         "    const long long np = n >> 1;\n"
         "    for (long long q = t; q < np; q += nt) {\n"
         "      const long long i = 2 * q;\n";
    for (int k = 0; k < kMapMaxInputs; ++k) {
        const std::string ks = std::to_string(k);
        if (k < nin) s += "      const " + T2 + " a" + ks + " = ((const " + T2 + "*)p" + ks + ")[q];\n";
        else s += "      const " + T2 + " a" + ks + " = {" + zero + ", " + zero + "};\n";
    }
    s += "      const " + T + " v0 = hyd_elem(i";
    for (int k = 0; k < kMapMaxInputs; ++k) s += ", a" + std::to_string(k) + ".x";
    s += ");\n      const " + T + " v1 = hyd_elem(i + 1";
    for (int k = 0; k < kMapMaxInputs; ++k) s += ", a" + std::to_string(k) + ".y";
    s += ");\n"
         "      if (out) { " + T2 + " w; w.x = v0; w.y = v1; ((" + T2 + "*)out)[q] = w; }\n"
         "      acc += (" + A + ")v0;\n"
         "      acc += (" + A + ")v1;\n"
         "    }\n"
         "    if (t == 0 && (n & 1)) {\n"
         "      const long long i = n - 1;\n"
         "      const " + T + " v = hyd_elem(i";
    for (int k = 0; k < kMapMaxInputs; ++k) s += k < nin ? ", p" + std::to_string(k) + "[i]" : ", " + zero;
    s += ");\n"
         "      if (out) out[i] = v;\n"
         "      acc += (" + A + ")v;\n"
         "    }\n"
         "  } else {\n"
         "    for (long long i = t; i < n; i += nt) {\n"
         "      const " + T + " v = hyd_elem(i";
    for (int k = 0; k < kMapMaxInputs; ++k) s += k < nin ? ", p" + std::to_string(k) + "[i]" : ", " + zero;
    s += ");\n"
         "      if (out) out[i] = v;\n"
         "      acc += (" + A + ")v;\n"
         "    }\n"
         "  }\n"
         "  if (sum == 0) return;\n"
         // fixed shuffle tree per warp, warps in order per block, blocks in order by the last block
         "  __shared__ " + A + " wsum[8];\n"
         "  __shared__ bool last;\n"
         "  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);\n"
         "  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = acc;\n"
         "  __syncthreads();\n"
         "  if (threadIdx.x == 0) {\n"
         "    " + A + " b = 0;\n"
         "    for (int w = 0; w < 8; ++w) b += wsum[w];\n"
         "    partials[blockIdx.x] = b;\n"
         "    __threadfence();\n"
         "    last = atomicAdd(counter, 1u) == gridDim.x - 1;\n"
         "  }\n"
         "  __syncthreads();\n"
         "  if (last && threadIdx.x == 0) {\n"
         "    __threadfence();\n"
         "    " + A + " s = 0;\n"
         "    for (unsigned b = 0; b < gridDim.x; ++b) s += __ldcg(partials + b);\n"
         "    *sum = s;\n"
         "    *counter = 0u;\n"
         "  }\n"
         "}\n";
    return s;
}

struct MapKernel {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kern = nullptr;
};
static std::map<std::tuple<int, int, bool, std::string>, MapKernel> g_map_kernels;

static int compile_map(Device* d, const std::string& body, int nin, bool i64, MapKernel* out) {
    std::lock_guard<std::mutex> lock(g_jit_mu);
    auto key = std::make_tuple(d->id, nin, i64, body);
    auto it = g_map_kernels.find(key);
    if (it != g_map_kernels.end()) {
        *out = it->second;
        return HYD_CUDA_OK;
    }
    if (!load_nvrtc_locked()) return set_error(HYD_CUDA_ERR_UNSUPPORTED, "map_f64: NVRTC library not found");
    int major = 0, minor = 0;
    HYD_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, d->id));
    HYD_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, d->id));
    const std::string src = map_source(body, nin, i64);
    nvrtcProgram prog = nullptr;
    if (g_nvrtc.create(&prog, src.c_str(), "hyd_map.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        return set_error(HYD_CUDA_ERR_CUDA, "map_f64: nvrtcCreateProgram failed");
    const std::string arch = "--gpu-architecture=sm_" + std::to_string(major) + std::to_string(minor);
    const char* opts[] = {arch.c_str(), "--fmad=false", "--std=c++17"};
    const nvrtcResult cr = g_nvrtc.compile(prog, 3, opts);
    if (cr != NVRTC_SUCCESS) {
        size_t n = 0;
        g_nvrtc.log_size(prog, &n);
        std::string log(n, '\0');
        if (n) g_nvrtc.log(prog, &log[0]);
        g_nvrtc.destroy(&prog);
        return set_error(HYD_CUDA_ERR_INVALID, "map_f64: the element body does not compile: %.400s", log.c_str());
    }
    size_t cn = 0;
    g_nvrtc.cubin_size(prog, &cn);
    std::vector<char> cubin(cn);
    g_nvrtc.cubin(prog, cubin.data());
    g_nvrtc.destroy(&prog);
    MapKernel mk;
    HYD_CUDA_TRY(cudaLibraryLoadData(&mk.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
    const cudaError_t ke = cudaLibraryGetKernel(&mk.kern, mk.lib, "hyd_map_kernel");
    if (ke != cudaSuccess) {
        cudaLibraryUnload(mk.lib);
        return set_error(HYD_CUDA_ERR_CUDA, "map_f64: %s", cudaGetErrorString(ke));
    }
    g_map_kernels[key] = mk;
    *out = mk;
    return HYD_CUDA_OK;
}

void release_map_kernels() {
    std::lock_guard<std::mutex> lock(g_jit_mu);
    for (auto& kv : g_map_kernels) cudaLibraryUnload(kv.second.lib);
    g_map_kernels.clear();
}

}  // namespace hyd

using namespace hyd;

template <class T>
static int map_launch(const char* body, const T* const* inputs, int ninputs, int64_t n, T* out, T* sum,
                      void* stream, const char* what) {
    HYD_CHECK_ARG(body != nullptr && *body, "%s: empty element body", what);
    HYD_CHECK_ARG(ninputs >= 0 && ninputs <= kMapMaxInputs, "%s: 0..%d inputs", what, kMapMaxInputs);
    HYD_CHECK_ARG(n >= 0, "%s: negative length", what);
    HYD_CHECK_ARG(ninputs == 0 || inputs != nullptr, "%s: null input table", what);
    for (int k = 0; k < ninputs; ++k) HYD_CHECK_ARG(n == 0 || inputs[k] != nullptr, "%s: null input %d", what, k);
    cudaStream_t s = as_stream(stream);
    Device* d = nullptr;
    HYD_TRY(device(&d));
    MapKernel mk;
    // compile errors surface even for n == 0
    HYD_TRY(compile_map(d, body, ninputs, std::is_integral<T>::value, &mk));
    if (n == 0) {
        if (sum) HYD_CUDA_TRY(cudaMemsetAsync(sum, 0, sizeof(T), s));
        return HYD_CUDA_OK;
    }
    // 2: every pointer 32-byte aligned (256-bit loads and stores); 1: 16-byte
    // aligned (128-bit); 0: scalar.  A null `out` counts as aligned, so a
    // reduction alone takes the same path, and gives the same bits, as with out.
    bool vec = (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    bool vec32 = (reinterpret_cast<uintptr_t>(out) & 31) == 0;
    const T* p[kMapMaxInputs] = {nullptr};
    for (int k = 0; k < ninputs; ++k) {
        p[k] = inputs[k];
        vec = vec && (reinterpret_cast<uintptr_t>(p[k]) & 15) == 0;
        vec32 = vec32 && (reinterpret_cast<uintptr_t>(p[k]) & 31) == 0;
    }
    const int64_t pairs = (n + 1) / 2;
    int64_t grid = (pairs + kMapThreads - 1) / kMapThreads;
    const int64_t cap = (int64_t)d->sm_count * 8;
    if (grid > cap) grid = cap;
    unsigned* counters = nullptr;
    void* scratch = nullptr;
    HYD_TRY(workspace(s, (size_t)grid * sizeof(T), &counters, &scratch));
    unsigned* counter = counters + 200;  // reset by the kernel's last block
    void* partials = scratch;
    long long nn = n;
    int v = vec32 ? 2 : (vec ? 1 : 0);
    void* args[kMapMaxInputs + 6];
    for (int k = 0; k < kMapMaxInputs; ++k) args[k] = &p[k];
    args[kMapMaxInputs + 0] = &nn;
    args[kMapMaxInputs + 1] = &out;
    args[kMapMaxInputs + 2] = &partials;
    args[kMapMaxInputs + 3] = &counter;
    args[kMapMaxInputs + 4] = &sum;
    args[kMapMaxInputs + 5] = &v;
    HYD_CUDA_TRY(cudaLaunchKernel((const void*)mk.kern, dim3((unsigned)grid), dim3(kMapThreads), args, 0, s));
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_map_f64(const char* body, const double* const* inputs, int ninputs, int64_t n, double* out,
                                double* sum, void* stream) {
    return map_launch<double>(body, inputs, ninputs, n, out, sum, stream, "map_f64");
}

extern "C" int hyd_cuda_map_i64(const char* body, const int64_t* const* inputs, int ninputs, int64_t n,
                                int64_t* out, int64_t* sum, void* stream) {
    return map_launch<long long>(body, reinterpret_cast<const long long* const*>(inputs), ninputs, n,
                                 reinterpret_cast<long long*>(out), reinterpret_cast<long long*>(sum), stream,
                                 "map_i64");
}
