// selftest.cu -- device probes that the tests and the bench use, with no
// counterpart in the reference:
//   * hyd_cuda_probe_fp64_rate: the FP64 unit's issue rate on this device,
//     measured by the caller with CUDA events around a kernel of independent
//     DFMA chains.  It is the denominator of the roofline of the kernels that
//     the FP64 unit bounds (the stencils, jacobi_1d, Gray-Scott, map_chain).
//   * hyd_cuda_selftest_timeout: makes one of the runtime's bounded device
//     waits run out, on a wait that nothing will ever satisfy, so that the
//     timeout path (error bit, HYD_CUDA_ERR_TIMEOUT from hyd_cuda_check, the
//     context still usable) is exercised without hanging or faulting the GPU.
#include "hyd_common.cuh"

namespace hyd {

constexpr int kRateThreads = 256;
constexpr int kRateBlocksPerSM = 4;
constexpr int kRateChains = 8;

// kRateChains independent fma chains per thread: a <- a * m + c with |m| < 1,
// so the values stay normal and bounded; the sum is stored so that nothing is
// optimised away.
__global__ void __launch_bounds__(kRateThreads) fp64_rate_kernel(int64_t iters, double* sink) {
    double a[kRateChains];
#pragma unroll
    for (int k = 0; k < kRateChains; ++k) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    const double m = 0.999999, c = 1e-7;
    for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < kRateChains; ++k) a[k] = fma(a[k], m, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kRateChains; ++k) s += a[k];
    if (s == 12345.678) sink[0] = s;  // never true; keeps the chains live
    if (blockIdx.x == 0 && threadIdx.x == 0) sink[1] = s;
}

// Timeout self-test 0: one thread waits on an mbarrier (arrival count 1) that
// nothing arrives at, through the bounded wait the TMA kernels use.
__global__ void selftest_mbar_timeout_kernel(unsigned limit, unsigned* err) {
    __shared__ __align__(8) unsigned long long bar;
    const unsigned addr = (unsigned)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) {
        mbar_init(addr, 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (!mbar_wait_bounded(addr, 0u, limit)) raise_error(err, ERRBIT_TIMEOUT);
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(addr) : "memory");
    }
}

// Timeout self-test 1: one warp looks back over 32 tile status words that are
// all zero ("nothing published"), through the wait the scans use.
__global__ void selftest_lookback_timeout_kernel(const TileWord* words, unsigned limit, unsigned* err) {
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < 32) {
        unsigned long long bits;
        const unsigned f = lookback_wait_words(words, 31, lane, bits, limit);
        if (f == 0u && lane == 0) raise_error(err, ERRBIT_TIMEOUT);
    }
}

}  // namespace hyd

using namespace hyd;

extern "C" int hyd_cuda_probe_fp64_rate(int64_t iters, double* sink, int64_t* fma_count, void* stream) {
    HYD_CHECK_ARG(iters > 0 && iters <= (int64_t)1 << 30, "probe_fp64_rate: iters outside 1..2^30");
    HYD_CHECK_ARG(sink != nullptr, "probe_fp64_rate: null sink (two device doubles)");
    Device* d = nullptr;
    HYD_TRY(device(&d));
    const int64_t blocks = (int64_t)d->sm_count * kRateBlocksPerSM;
    fp64_rate_kernel<<<(unsigned)blocks, kRateThreads, 0, as_stream(stream)>>>(iters, sink);
    if (fma_count) *fma_count = blocks * kRateThreads * kRateChains * iters;
    return launch_check("probe_fp64_rate");
}

extern "C" int hyd_cuda_selftest_timeout(int which, uint32_t poll_limit, void* stream) {
    HYD_CHECK_ARG(which == 0 || which == 1, "selftest_timeout: which is 0 (mbarrier) or 1 (look-back)");
    HYD_CHECK_ARG(poll_limit >= 1 && poll_limit <= (1u << 20), "selftest_timeout: poll limit outside 1..2^20");
    Device* d = nullptr;
    HYD_TRY(device(&d));
    cudaStream_t s = as_stream(stream);
    if (which == 0) {
        selftest_mbar_timeout_kernel<<<1, 32, 0, s>>>(poll_limit, d->d_err);
    } else {
        void* scratch = nullptr;
        HYD_TRY(workspace(s, 32 * sizeof(TileWord), nullptr, &scratch));
        HYD_CUDA_TRY(cudaMemsetAsync(scratch, 0, 32 * sizeof(TileWord), s));
        selftest_lookback_timeout_kernel<<<1, 32, 0, s>>>(static_cast<const TileWord*>(scratch), poll_limit,
                                                          d->d_err);
    }
    return launch_check("selftest_timeout");
}
