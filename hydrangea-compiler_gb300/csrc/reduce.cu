// reduce.cu -- deterministic fp64 reductions: the fused
// `reduce (+) 0.0 (zipwith (*) xs ys)` (dot) and `reduce (+) 0.0 xs` (sum).
//
// Replaces the parallel reduction template of the reference C backend
// (CodegenC.hs:1328-1353; emitted `omp parallel for simd reduction(+:acc)`,
// README.md:25-33) for the 1-D reduce_generate of Lowering.hs:771-804.
//
// Design (HBM-bound streaming reduction, one launch):
//  * a fixed grid of 2 blocks x 512 threads per SM; thread t owns the 32-byte
//    vectors t, t+S, t+2S, ... (S = total threads) and keeps two independent
//    sets of four fp64 accumulators, so four 256-bit loads are in flight per
//    thread and the DFMA latency chains stay short;
//  * per-thread order, the xor-butterfly warp tree, the cross-warp tree and the
//    final combine are all fixed, so a given (n, device) always produces the
//    same bits (the C backend's result instead depends on the thread count);
//  * the block partials go to per-stream scratch; the last block to finish
//    (completion counter) sums them in index order and resets the counter,
//    so no second launch and no memset are needed per call.
// Products are accumulated with fma (one rounding per element instead of the
// C backend's two); the tolerance against the C backend is relative 1e-12.
#include "hyd_common.cuh"

namespace hyd {

constexpr int kRedThreads = 512;
constexpr int kRedBlocksPerSM = 2;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-order block reduction; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (warp == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// Last-block combine of the per-block partials, in index order.
__device__ __forceinline__ void finish_partials(double bsum, double* partials, unsigned* counter,
                                                double* out, double* sh) {
    __shared__ bool is_last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bsum;
        __threadfence();
        unsigned ticket = atomicAdd(counter, 1u);
        is_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double v = 0.0;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x)
        v += *((volatile double*)&partials[i]);
    double total = block_sum(v, sh);
    if (threadIdx.x == 0) {
        *out = total;
        *counter = 0u;  // leave the counter ready for the next launch
    }
}

template <bool kDot, bool kVec>
__global__ void __launch_bounds__(kRedThreads, kRedBlocksPerSM)
    reduce_f64_kernel(const double* __restrict__ xs, const double* __restrict__ ys, int64_t n,
                      double* partials, unsigned* counter, double* out) {
    __shared__ double sh[32];
    const int64_t S = (int64_t)gridDim.x * blockDim.x;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    double b0 = 0.0, b1 = 0.0, b2 = 0.0, b3 = 0.0;
    int64_t tail_start = 0;
    if (kVec) {
        const int64_t nv = n >> 2;  // 32-byte vectors
        int64_t v = t;
        for (; v + S < nv; v += 2 * S) {
            f64x4 x0 = ldg_stream_f64x4(xs + 4 * v);
            f64x4 x1 = ldg_stream_f64x4(xs + 4 * (v + S));
            if (kDot) {
                f64x4 y0 = ldg_stream_f64x4(ys + 4 * v);
                f64x4 y1 = ldg_stream_f64x4(ys + 4 * (v + S));
                a0 = fma(x0.x, y0.x, a0); a1 = fma(x0.y, y0.y, a1);
                a2 = fma(x0.z, y0.z, a2); a3 = fma(x0.w, y0.w, a3);
                b0 = fma(x1.x, y1.x, b0); b1 = fma(x1.y, y1.y, b1);
                b2 = fma(x1.z, y1.z, b2); b3 = fma(x1.w, y1.w, b3);
            } else {
                a0 += x0.x; a1 += x0.y; a2 += x0.z; a3 += x0.w;
                b0 += x1.x; b1 += x1.y; b2 += x1.z; b3 += x1.w;
            }
        }
        if (v < nv) {
            f64x4 x0 = ldg_stream_f64x4(xs + 4 * v);
            if (kDot) {
                f64x4 y0 = ldg_stream_f64x4(ys + 4 * v);
                a0 = fma(x0.x, y0.x, a0); a1 = fma(x0.y, y0.y, a1);
                a2 = fma(x0.z, y0.z, a2); a3 = fma(x0.w, y0.w, a3);
            } else {
                a0 += x0.x; a1 += x0.y; a2 += x0.z; a3 += x0.w;
            }
        }
        tail_start = nv * 4;
    }
    // scalar remainder (or the whole array when the pointers are not 32-byte aligned)
    for (int64_t i = tail_start + t; i < n; i += S) {
        if (kDot) a0 = fma(xs[i], ys[i], a0);
        else a0 += xs[i];
    }
    double v = ((a0 + a1) + (a2 + a3)) + ((b0 + b1) + (b2 + b3));
    double bsum = block_sum(v, sh);
    __syncthreads();
    finish_partials(bsum, partials, counter, out, sh);
}

static int reduce_launch(bool dot, const double* xs, const double* ys, int64_t n, double* out,
                         cudaStream_t stream) {
    Device* d = nullptr;
    HYD_TRY(device(&d));
    const int64_t units = (n + 3) / 4;
    int64_t blocks = (int64_t)d->sm_count * kRedBlocksPerSM;
    int64_t want = (units + 2LL * kRedThreads - 1) / (2LL * kRedThreads);
    if (want < blocks) blocks = want < 1 ? 1 : want;
    unsigned* counters = nullptr;
    void* scratch = nullptr;
    HYD_TRY(workspace(stream, sizeof(double) * (size_t)blocks, &counters, &scratch));
    double* partials = static_cast<double*>(scratch);
    unsigned* counter = counters + (dot ? 0 : 1);
    const bool vec = ((reinterpret_cast<uintptr_t>(xs) | (dot ? reinterpret_cast<uintptr_t>(ys) : 0)) & 31) == 0;
    dim3 grid((unsigned)blocks), block(kRedThreads);
    if (dot) {
        if (vec) reduce_f64_kernel<true, true><<<grid, block, 0, stream>>>(xs, ys, n, partials, counter, out);
        else reduce_f64_kernel<true, false><<<grid, block, 0, stream>>>(xs, ys, n, partials, counter, out);
    } else {
        if (vec) reduce_f64_kernel<false, true><<<grid, block, 0, stream>>>(xs, xs, n, partials, counter, out);
        else reduce_f64_kernel<false, false><<<grid, block, 0, stream>>>(xs, xs, n, partials, counter, out);
    }
    return launch_check(dot ? "dot_f64" : "sum_f64");
}

}  // namespace hyd

using namespace hyd;

extern "C" int hyd_cuda_dot_f64(const double* xs, const double* ys, int64_t n, double* out,
                                void* stream) {
    HYD_CHECK_ARG(n >= 0, "dot_f64: negative length %lld", (long long)n);
    HYD_CHECK_ARG(out != nullptr, "dot_f64: null output");
    HYD_CHECK_ARG(n == 0 || (xs != nullptr && ys != nullptr), "dot_f64: null input");
    return reduce_launch(true, xs, ys, n, out, as_stream(stream));
}

extern "C" int hyd_cuda_sum_f64(const double* xs, int64_t n, double* out, void* stream) {
    HYD_CHECK_ARG(n >= 0, "sum_f64: negative length %lld", (long long)n);
    HYD_CHECK_ARG(out != nullptr, "sum_f64: null output");
    HYD_CHECK_ARG(n == 0 || xs != nullptr, "sum_f64: null input");
    return reduce_launch(false, xs, nullptr, n, out, as_stream(stream));
}

// ---------------------------------------------------------------------------
// Allocation-free dot product.
//
// Some callers cannot allocate device memory at the point where they need a
// reduction: a latency-critical serving or real-time loop where cudaMalloc
// (and the cudaFree that pairs with it) may synchronize the device and stall
// work on other streams; a process whose device memory was reserved up front
// by another allocator or capped by a memory policy, where a fresh cudaMalloc
// can fail at an arbitrary moment; an embedding host that requires a fixed
// footprint after start-up.  hyd_cuda_dot_f64 takes its scratch (per-CTA
// partials and a completion counter) from a per-stream workspace that the
// runtime allocates on first use, so it is not usable there.
//
// hyd_cuda_dot_f64_noalloc runs the same kernel with its scratch in the
// file-scope array below instead.  The array is fixed at load time, so every
// GPU that loads this library holds these bytes until the process exits.  Its
// size bounds the launch: kNoAllocMaxBlocks CTAs (two per SM on any GPU with
// up to 1024 SMs); a launch that would need more is rejected.
namespace hyd {

constexpr int kNoAllocMaxBlocks = 2048;
constexpr size_t kNoAllocCounterBytes = 256;
constexpr size_t kNoAllocScratchBytes = kNoAllocCounterBytes + sizeof(double) * kNoAllocMaxBlocks;

static __device__ __align__(256) unsigned char g_dot_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_dot_noalloc_scratch, looked up once per device with that
// device current.  In host code the symbol itself is only a host-side stand-in,
// never a device address, so kernels must be given this pointer.
static std::mutex g_noalloc_mu;
static unsigned char* g_noalloc_ptr[64] = {nullptr};
static int g_noalloc_sms[64] = {0};

static int noalloc_setup(int dev, unsigned char** scratch, int* sms) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_dot_noalloc_scratch);
        if (e != cudaSuccess)
            return set_error(HYD_CUDA_ERR_CUDA, "dot_f64_noalloc: cudaGetSymbolAddress failed: %s",
                             cudaGetErrorString(e));
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess)
            return set_error(HYD_CUDA_ERR_CUDA, "dot_f64_noalloc: SM count query failed: %s",
                             cudaGetErrorString(e));
        g_noalloc_sms[dev] = n;
        g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *scratch = g_noalloc_ptr[dev];
    *sms = g_noalloc_sms[dev];
    return HYD_CUDA_OK;
}

}  // namespace hyd

extern "C" int hyd_cuda_dot_f64_noalloc(const double* xs, const double* ys, int64_t n, double* out,
                                        void* stream) {
    HYD_CHECK_ARG(n >= 0, "dot_f64_noalloc: negative length %lld", (long long)n);
    HYD_CHECK_ARG(out != nullptr, "dot_f64_noalloc: null output");
    HYD_CHECK_ARG(n == 0 || (xs != nullptr && ys != nullptr), "dot_f64_noalloc: null input");
    int dev = 0;
    HYD_CUDA_TRY(cudaGetDevice(&dev));
    HYD_CHECK_ARG(dev >= 0 && dev < 64, "dot_f64_noalloc: device ordinal %d beyond 63", dev);
    unsigned char* scratch = nullptr;
    int sms = 0;
    HYD_TRY(noalloc_setup(dev, &scratch, &sms));
    // Same grid rule as hyd_cuda_dot_f64, so both give the same bits.
    const int64_t units = (n + 3) / 4;
    int64_t blocks = (int64_t)sms * kRedBlocksPerSM;
    const int64_t want = (units + 2LL * kRedThreads - 1) / (2LL * kRedThreads);
    if (want < blocks) blocks = want < 1 ? 1 : want;
    if (blocks > kNoAllocMaxBlocks)
        return set_error(HYD_CUDA_ERR_UNSUPPORTED,
                         "dot_f64_noalloc: needs %lld CTAs of scratch but the static scratch holds %d",
                         (long long)blocks, kNoAllocMaxBlocks);
    unsigned* counter = reinterpret_cast<unsigned*>(scratch);
    double* partials = reinterpret_cast<double*>(scratch + kNoAllocCounterBytes);
    cudaStream_t st = as_stream(stream);
    // The array keeps whatever the previous call left; the counter must start at 0.
    HYD_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned), st));
    const bool vec = ((reinterpret_cast<uintptr_t>(xs) | reinterpret_cast<uintptr_t>(ys)) & 31) == 0;
    if (vec)
        reduce_f64_kernel<true, true><<<(unsigned)blocks, kRedThreads, 0, st>>>(xs, ys, n, partials, counter, out);
    else
        reduce_f64_kernel<true, false><<<(unsigned)blocks, kRedThreads, 0, st>>>(xs, ys, n, partials, counter, out);
    return launch_check("dot_f64_noalloc");
}
