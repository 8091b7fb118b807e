// histogram.cu -- scatter (+): the fused weighted histogram
//   scatter (+) (fill [B] 0) (map (x % B) data) (map (x * x) data)
// and the unfused scatter-add over materialised routes/values.
//
// Replaces the reference C backend's privatized scatter template
// (CodegenC.hs:1119-1288: an nthreads x B grid of private bins, accumulate,
// merge in thread order) and its atomic template (CodegenC.hs:1084-1118),
// chosen by Parallelize.hs:466-503.  On the GPU the private copies live in
// on-chip memory instead of DRAM:
//  * SMEM_WARP   one copy of the B bins per warp in shared memory, so atomics
//                only contend inside a warp; copies merged per block into the
//                destination with one global atomic per non-zero bin;
//  * SMEM_BLOCK  one copy per block (more bins fit);
//  * CLUSTER     the B bins are spread over the shared memory of a thread-block
//                cluster (up to 16 CTAs); each element is added into the owning
//                CTA's slice with a distributed-shared-memory reduction
//                (`red.shared::cluster.add.u64`); B up to ~3M bins on chip;
//  * GLOBAL      `red.global.add` straight into the destination (L2 atomics),
//                the fallback when the bins exceed the cluster's memory.
// int64 adds wrap and commute, so every strategy gives the bit-identical
// result of the C backend.  The input is streamed once with 256-bit
// non-allocating loads; that read is the roofline (8 bytes per element).
#include "hyd_common.cuh"

namespace hyd {

constexpr int kHistThreads = 512;

// Element sources: produce (route, value) for element i.
struct WeightedHistSource {
    const int64_t* data;
    DivMod64 dm;
    static constexpr bool kVecAligned = true;
    __device__ __forceinline__ void one(int64_t i, long long& bin, unsigned long long& val) const {
        long long x = data[i];
        bin = dm.rem(x);
        val = (unsigned long long)x * (unsigned long long)x;
    }
    __device__ __forceinline__ void four(int64_t v, long long bin[4], unsigned long long val[4]) const {
        u64x4 q = ldg_stream_u64x4(data + 4 * v);
        long long x[4] = {(long long)q.x, (long long)q.y, (long long)q.z, (long long)q.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            bin[k] = dm.rem(x[k]);
            val[k] = (unsigned long long)x[k] * (unsigned long long)x[k];
        }
    }
};

struct ScatterI64Source {
    const int64_t* idx;
    const int64_t* vals;
    __device__ __forceinline__ void one(int64_t i, long long& bin, unsigned long long& val) const {
        bin = idx[i];
        val = (unsigned long long)vals[i];
    }
    __device__ __forceinline__ void four(int64_t v, long long bin[4], unsigned long long val[4]) const {
        u64x4 a = ldg_stream_u64x4(idx + 4 * v);
        u64x4 b = ldg_stream_u64x4(vals + 4 * v);
        bin[0] = (long long)a.x; bin[1] = (long long)a.y; bin[2] = (long long)a.z; bin[3] = (long long)a.w;
        val[0] = b.x; val[1] = b.y; val[2] = b.z; val[3] = b.w;
    }
};

// Iterate this thread's elements: 32-byte groups t, t+S, ... (two in flight),
// then the scalar remainder.  f(bin, val) is called per element.
template <class Src, class F>
__device__ __forceinline__ void for_each_element(const Src& src, int64_t n, bool vec, F f) {
    const int64_t S = (int64_t)gridDim.x * blockDim.x;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t tail = 0;
    if (vec) {
        const int64_t nv = n >> 2;
        int64_t v = t;
        for (; v + S < nv; v += 2 * S) {
            long long b0[4], b1[4];
            unsigned long long v0[4], v1[4];
            src.four(v, b0, v0);
            src.four(v + S, b1, v1);
#pragma unroll
            for (int k = 0; k < 4; ++k) f(b0[k], v0[k]);
#pragma unroll
            for (int k = 0; k < 4; ++k) f(b1[k], v1[k]);
        }
        if (v < nv) {
            long long b0[4];
            unsigned long long v0[4];
            src.four(v, b0, v0);
#pragma unroll
            for (int k = 0; k < 4; ++k) f(b0[k], v0[k]);
        }
        tail = nv * 4;
    }
    for (int64_t i = tail + t; i < n; i += S) {
        long long b;
        unsigned long long v;
        src.one(i, b, v);
        f(b, v);
    }
}

// ---- shared-memory privatized (per-warp or per-block copies) --------------
template <class Src>
__global__ void __launch_bounds__(kHistThreads, 2)
    hist_smem_kernel(Src src, int64_t n, bool vec, int bins, int copies,
                     unsigned long long* __restrict__ hist, unsigned* err) {
    extern __shared__ unsigned long long sh_bins[];
    const int total = copies * bins;
    for (int i = threadIdx.x; i < total; i += blockDim.x) sh_bins[i] = 0ULL;
    __syncthreads();
    unsigned long long* mine = sh_bins + ((threadIdx.x >> 5) % copies) * bins;
    bool bad = false;
    for_each_element(src, n, vec, [&](long long b, unsigned long long v) {
        if ((unsigned long long)b < (unsigned long long)bins) atomicAdd(&mine[b], v);
        else bad = true;
    });
    __syncthreads();
    for (int b = threadIdx.x; b < bins; b += blockDim.x) {
        unsigned long long s = 0;
        for (int c = 0; c < copies; ++c) s += sh_bins[c * bins + b];
        if (s) atomicAdd(&hist[b], s);
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// ---- cluster distributed shared memory -------------------------------------
__device__ __forceinline__ unsigned cluster_ctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned map_shared_rank(unsigned local_addr, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void dsmem_red_add_u64(unsigned cluster_addr, unsigned long long v) {
    asm volatile("red.shared::cluster.add.u64 [%0], %1;" ::"r"(cluster_addr), "l"(v) : "memory");
}

template <class Src>
__global__ void __launch_bounds__(kHistThreads, 2)
    hist_cluster_kernel(Src src, int64_t n, bool vec, long long bins, int per_cta_shift,
                        unsigned long long* __restrict__ hist, unsigned* err) {
    extern __shared__ unsigned long long sh_bins[];
    const int per_cta = 1 << per_cta_shift;
    for (int i = threadIdx.x; i < per_cta; i += blockDim.x) sh_bins[i] = 0ULL;
    cluster_sync_all();
    const unsigned base = (unsigned)__cvta_generic_to_shared(sh_bins);
    bool bad = false;
    for_each_element(src, n, vec, [&](long long b, unsigned long long v) {
        if ((unsigned long long)b < (unsigned long long)bins) {
            unsigned owner = (unsigned)(b >> per_cta_shift);
            unsigned local = (unsigned)(b & (per_cta - 1));
            dsmem_red_add_u64(map_shared_rank(base + local * 8u, owner), v);
        } else {
            bad = true;
        }
    });
    cluster_sync_all();  // every remote add into this CTA's slice has landed
    const long long first = (long long)cluster_ctarank() << per_cta_shift;
    for (int i = threadIdx.x; i < per_cta; i += blockDim.x) {
        long long g = first + i;
        unsigned long long s = sh_bins[i];
        if (g < bins && s) atomicAdd(&hist[g], s);
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// ---- global atomics --------------------------------------------------------
template <class Src>
__global__ void __launch_bounds__(kHistThreads, 2)
    hist_global_kernel(Src src, int64_t n, bool vec, long long bins,
                       unsigned long long* __restrict__ hist, unsigned* err) {
    bool bad = false;
    for_each_element(src, n, vec, [&](long long b, unsigned long long v) {
        if ((unsigned long long)b < (unsigned long long)bins) atomicAdd(&hist[b], v);
        else bad = true;
    });
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// ---- host side --------------------------------------------------------------
struct HistPlan {
    int strategy;
    int copies;       // SMEM_*: copies per block
    int cluster;      // CLUSTER: CTAs per cluster
    int shift;        // CLUSTER: log2(bins per CTA)
    size_t smem;      // dynamic shared memory bytes
    int blocks;
};

static int log2_ceil(long long v) {
    int s = 0;
    while ((1LL << s) < v) ++s;
    return s;
}

// Shared memory one CTA may use for bins while keeping 2 CTAs per SM.
static size_t smem_budget(const Device* d) {
    size_t optin = (size_t)d->max_smem_optin;
    return optin / 2 - 1024;
}

static int plan_hist(const Device* d, long long bins, int strategy, HistPlan* p) {
    const size_t bytes = (size_t)bins * 8;
    const size_t budget = smem_budget(d);
    const size_t optin = (size_t)d->max_smem_optin;
    const int warps = kHistThreads / 32;
    if (strategy == HYD_SCATTER_AUTO) {
        // Default choice for the (bins) class; measured alternatives are kept
        // selectable and recorded by the autotuner.
        if (bytes * 4 <= budget) strategy = HYD_SCATTER_SMEM_WARP;
        else if (bytes <= budget) strategy = HYD_SCATTER_SMEM_BLOCK;
        else if (bytes <= optin * 16 / 2) strategy = HYD_SCATTER_CLUSTER;
        else strategy = HYD_SCATTER_GLOBAL;
    }
    p->strategy = strategy;
    p->copies = 1;
    p->cluster = 1;
    p->shift = 0;
    p->smem = 0;
    switch (strategy) {
        case HYD_SCATTER_SMEM_WARP: {
            if (bytes > budget) return set_error(HYD_CUDA_ERR_UNSUPPORTED, "SMEM_WARP: %lld bins exceed shared memory", bins);
            int c = (int)(budget / bytes);
            p->copies = c > warps ? warps : c;
            p->smem = bytes * p->copies;
            p->blocks = d->sm_count * 2;
            break;
        }
        case HYD_SCATTER_SMEM_BLOCK:
            if (bytes > optin - 1024) return set_error(HYD_CUDA_ERR_UNSUPPORTED, "SMEM_BLOCK: %lld bins exceed shared memory", bins);
            p->smem = bytes;
            p->blocks = d->sm_count * (bytes <= budget ? 2 : 1);
            break;
        case HYD_SCATTER_CLUSTER: {
            // smallest cluster whose slices fit; slices are powers of two
            int cl = 2;
            while (cl <= 16 && ((size_t)8 << log2_ceil((bins + cl - 1) / cl)) > budget) cl *= 2;
            if (cl > 16) {
                cl = 16;
                if (((size_t)8 << log2_ceil((bins + 15) / 16)) > optin - 1024)
                    return set_error(HYD_CUDA_ERR_UNSUPPORTED, "CLUSTER: %lld bins exceed 16 CTAs of shared memory", bins);
            }
            p->cluster = cl;
            p->shift = log2_ceil((bins + cl - 1) / cl);
            p->smem = (size_t)8 << p->shift;
            int per_sm = p->smem <= budget ? 2 : 1;
            p->blocks = (d->sm_count * per_sm / cl) * cl;
            if (p->blocks < cl) p->blocks = cl;
            break;
        }
        case HYD_SCATTER_GLOBAL:
            p->blocks = d->sm_count * 2;
            break;
        default:
            return set_error(HYD_CUDA_ERR_INVALID, "unknown scatter strategy %d", strategy);
    }
    return HYD_CUDA_OK;
}

template <class Src>
static int hist_launch(const Src& src, int64_t n, bool vec, long long bins, unsigned long long* hist,
                       int strategy, cudaStream_t stream, const char* what) {
    Device* d = nullptr;
    HYD_TRY(device(&d));
    HistPlan p;
    HYD_TRY(plan_hist(d, bins, strategy, &p));
    // Do not launch more CTAs than there are 32-byte groups to stream.
    int64_t groups = (n + 3) / 4;
    int64_t want = (groups + kHistThreads - 1) / kHistThreads;
    if (p.strategy != HYD_SCATTER_CLUSTER && want < p.blocks) p.blocks = want < 1 ? 1 : (int)want;
    switch (p.strategy) {
        case HYD_SCATTER_SMEM_WARP:
        case HYD_SCATTER_SMEM_BLOCK: {
            auto k = hist_smem_kernel<Src>;
            HYD_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem));
            k<<<p.blocks, kHistThreads, p.smem, stream>>>(src, n, vec, (int)bins, p.copies, hist, d->d_err);
            break;
        }
        case HYD_SCATTER_CLUSTER: {
            auto k = hist_cluster_kernel<Src>;
            HYD_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem));
            if (p.cluster > 8)
                HYD_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)p.blocks);
            cfg.blockDim = dim3(kHistThreads);
            cfg.dynamicSmemBytes = p.smem;
            cfg.stream = stream;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = (unsigned)p.cluster;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            HYD_CUDA_TRY(cudaLaunchKernelEx(&cfg, k, src, n, vec, bins, p.shift, hist, d->d_err));
            break;
        }
        case HYD_SCATTER_GLOBAL:
            hist_global_kernel<Src><<<p.blocks, kHistThreads, 0, stream>>>(src, n, vec, bins, hist, d->d_err);
            break;
    }
    return launch_check(what);
}

// Plain fp64 scatter-add (global atomics; order-dependent rounding).
__global__ void scatter_add_f64_kernel(const int64_t* __restrict__ idx, const double* __restrict__ vals,
                                       int64_t n, double* dst, int64_t dst_n, unsigned* err) {
    const int64_t S = (int64_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += S) {
        int64_t b = idx[i];
        if ((uint64_t)b < (uint64_t)dst_n) atomicAdd(&dst[b], vals[i]);
        else bad = true;
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

}  // namespace hyd

using namespace hyd;

extern "C" int hyd_cuda_weighted_histogram_i64(const int64_t* data, int64_t n, int64_t bins,
                                               int64_t* hist, int strategy, void* stream) {
    HYD_CHECK_ARG(n >= 0, "weighted_histogram: negative length %lld", (long long)n);
    HYD_CHECK_ARG(bins > 0, "weighted_histogram: bins must be positive (got %lld)", (long long)bins);
    HYD_CHECK_ARG(hist != nullptr, "weighted_histogram: null histogram");
    HYD_CHECK_ARG(n == 0 || data != nullptr, "weighted_histogram: null data");
    HYD_CHECK_ARG(strategy >= HYD_SCATTER_AUTO && strategy <= HYD_SCATTER_GLOBAL,
                  "weighted_histogram: unknown strategy %d", strategy);
    HYD_CHECK_ARG(bins <= (1LL << 31), "weighted_histogram: bins beyond 2^31 unsupported");
    if (n == 0) return HYD_CUDA_OK;
    WeightedHistSource src;
    src.data = data;
    src.dm.init(bins);
    bool vec = (reinterpret_cast<uintptr_t>(data) & 31) == 0;
    return hist_launch(src, n, vec, bins, reinterpret_cast<unsigned long long*>(hist), strategy,
                       as_stream(stream), "weighted_histogram_i64");
}

extern "C" int hyd_cuda_scatter_add_i64(const int64_t* idx, const int64_t* vals, int64_t n,
                                        int64_t* dst, int64_t dst_n, int strategy, void* stream) {
    HYD_CHECK_ARG(n >= 0, "scatter_add_i64: negative length");
    HYD_CHECK_ARG(dst_n > 0, "scatter_add_i64: empty destination");
    HYD_CHECK_ARG(dst != nullptr, "scatter_add_i64: null destination");
    HYD_CHECK_ARG(n == 0 || (idx != nullptr && vals != nullptr), "scatter_add_i64: null input");
    HYD_CHECK_ARG(strategy >= HYD_SCATTER_AUTO && strategy <= HYD_SCATTER_GLOBAL,
                  "scatter_add_i64: unknown strategy %d", strategy);
    HYD_CHECK_ARG(dst_n <= (1LL << 31), "scatter_add_i64: destination beyond 2^31 unsupported");
    if (n == 0) return HYD_CUDA_OK;
    ScatterI64Source src{idx, vals};
    bool vec = ((reinterpret_cast<uintptr_t>(idx) | reinterpret_cast<uintptr_t>(vals)) & 31) == 0;
    return hist_launch(src, n, vec, dst_n, reinterpret_cast<unsigned long long*>(dst), strategy,
                       as_stream(stream), "scatter_add_i64");
}

extern "C" int hyd_cuda_scatter_add_f64(const int64_t* idx, const double* vals, int64_t n,
                                        double* dst, int64_t dst_n, void* stream) {
    HYD_CHECK_ARG(n >= 0, "scatter_add_f64: negative length");
    HYD_CHECK_ARG(dst_n > 0 && dst != nullptr, "scatter_add_f64: empty or null destination");
    HYD_CHECK_ARG(n == 0 || (idx != nullptr && vals != nullptr), "scatter_add_f64: null input");
    if (n == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    int64_t want = (n + 255) / 256;
    int blocks = (int)(want < d->sm_count * 4 ? want : d->sm_count * 4);
    scatter_add_f64_kernel<<<blocks, 256, 0, as_stream(stream)>>>(idx, vals, n, dst, dst_n, d->d_err);
    return launch_check("scatter_add_f64");
}
