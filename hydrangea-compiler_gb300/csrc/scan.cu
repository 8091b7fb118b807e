// scan.cu -- scan / scan_inclusive / scanr / scanr_inclusive with (+), and
// segmented_reduce (+).
//
// Replaces the serial LoopFold of lowerScanFamily (Lowering.hs:3563-3612; the
// C backend never parallelises a fold, Parallelize.hs:517) and the
// LoopSegRedOuter loop of segmented_reduce (Lowering.hs:874-944,
// `schedule(dynamic)` per CodegenC.hs:1055-1057).
//
// int64: single-pass decoupled look-back (Merrill & Garland, "Single-pass
// Parallel Prefix Scan with Decoupled Look-back", 2016).  Tiles of 4096
// elements take their id from an atomic counter in launch order, so every
// predecessor a tile waits on has already started; a tile publishes its
// aggregate, a warp looks back 32 predecessors at a time, then publishes its
// inclusive prefix.  Every spin is bounded (error bit, no hang).  int64 adds
// wrap and commute, so the result is bit-identical to the serial C fold.
// One read and one write per element: 16 B/element of HBM traffic.
//
// float64: reduce-then-scan in three launches with a fixed combine order, so
// results are run-to-run reproducible.  A parallel prefix cannot reproduce the
// serial fold's roundings; the tolerance is |gpu - c| <= 1e-12 * prefix sum of
// |x| (stated in the tests).
//
// Reverse scans read and write index n-1-k for logical position k, exactly the
// ix the reference's lowering computes.
#include "hyd_common.cuh"

namespace hyd {

constexpr int kScanT = 512;
constexpr int kScanIPT = 8;
constexpr int kScanTile = kScanT * kScanIPT;  // 4096 (32 KiB of static shared memory for int64)
constexpr unsigned kSpinLimit = 1u << 22;

// --- block-wide exclusive scan of one value per thread (int64, wrapping) ------
template <class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* sh /*[32]*/, T& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? sh[lane] : T(0);
        T wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += y;
        }
        sh[lane] = wi - w;  // exclusive warp offsets
        if (lane == 31) sh[32] = wi;
    }
    __syncthreads();
    total = sh[32];
    T r = sh[warp] + incl - v;
    __syncthreads();
    return r;
}

// Tile load/store in blocked arrangement through shared memory: global
// accesses are coalesced, each thread then owns kScanIPT consecutive logical
// elements.  Logical position k maps to physical index (reverse ? n-1-k : k).
template <class T>
__device__ __forceinline__ void tile_load(const T* in, int64_t n, int64_t base, bool reverse, T* sh,
                                          T (&items)[kScanIPT]) {
    for (int i = threadIdx.x; i < kScanTile; i += kScanT) {
        const int64_t k = base + i;
        T v = T(0);
        if (k < n) v = in[reverse ? (n - 1 - k) : k];
        sh[i] = v;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) items[j] = sh[threadIdx.x * kScanIPT + j];
    __syncthreads();
}

template <class T>
__device__ __forceinline__ void tile_store(T* out, int64_t n, int64_t base, bool reverse, T* sh,
                                           const T (&items)[kScanIPT]) {
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) sh[threadIdx.x * kScanIPT + j] = items[j];
    __syncthreads();
    for (int i = threadIdx.x; i < kScanTile; i += kScanT) {
        const int64_t k = base + i;
        if (k < n) out[reverse ? (n - 1 - k) : k] = sh[i];
    }
}

// ---- int64 decoupled look-back ----------------------------------------------------
// Status per tile: flag (0 none, 1 aggregate, 2 inclusive prefix) + two values.
struct ScanStatus {
    unsigned* flag;
    long long* aggregate;
    long long* inclusive;
    unsigned* tile_counter;
};

__device__ __forceinline__ unsigned ld_volatile_u32(const unsigned* p) { return *(volatile const unsigned*)p; }
__device__ __forceinline__ long long ld_volatile_i64(const long long* p) { return *(volatile const long long*)p; }

__global__ void __launch_bounds__(kScanT) scan_i64_lookback_kernel(const long long* __restrict__ in,
                                                                    long long* __restrict__ out, int64_t n,
                                                                    long long init, bool reverse,
                                                                    bool inclusive, ScanStatus st,
                                                                    unsigned* err) {
    __shared__ long long sh_tile[kScanTile];
    __shared__ long long sh_scan[33];
    __shared__ unsigned sh_tile_id;
    __shared__ long long sh_prefix;
    if (threadIdx.x == 0) sh_tile_id = atomicAdd(st.tile_counter, 1u);
    __syncthreads();
    const unsigned tile = sh_tile_id;
    const int64_t base = (int64_t)tile * kScanTile;

    long long items[kScanIPT];
    tile_load(in, n, base, reverse, sh_tile, items);
    long long tsum = 0;
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) tsum += items[j];
    long long agg;
    const long long texcl = block_exclusive_scan(tsum, sh_scan, agg);

    // publish and look back (warp 0)
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        if (tile == 0) {
            if (lane == 0) {
                st.inclusive[0] = init + agg;
                __threadfence();
                *(volatile unsigned*)&st.flag[0] = 2u;
                sh_prefix = init;
            }
        } else {
            if (lane == 0) {
                st.aggregate[tile] = agg;
                __threadfence();
                *(volatile unsigned*)&st.flag[tile] = 1u;
            }
            long long running = 0;
            int64_t p = (int64_t)tile - 1;  // window covers p, p-1, ..., p-31
            bool done = false;
            unsigned spins = 0;
            while (!done) {
                const int64_t q = p - lane;
                unsigned f = q >= 0 ? ld_volatile_u32(&st.flag[q]) : 2u;
                // wait until every tile of the window has published something
                while (__any_sync(0xffffffffu, f == 0u)) {
                    if (++spins > kSpinLimit) break;
                    if (f == 0u) f = ld_volatile_u32(&st.flag[q]);
                }
                if (spins > kSpinLimit) {
                    if (lane == 0) raise_error(err, ERRBIT_TIMEOUT);
                    break;
                }
                __threadfence();
                const unsigned incl_mask = __ballot_sync(0xffffffffu, f == 2u);
                // nearest predecessor with an inclusive prefix (lowest lane)
                const int stop = incl_mask ? (__ffs(incl_mask) - 1) : 32;
                long long v = 0;
                if (lane < stop && q >= 0) v = ld_volatile_i64(&st.aggregate[q]);
                if (lane == stop && q >= 0) v = ld_volatile_i64(&st.inclusive[q]);
                if (lane == stop && q < 0) v = init;  // before tile 0: the fold's initial value
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                running += v;
                if (stop < 32) done = true;
                p -= 32;
            }
            if (lane == 0) {
                st.inclusive[tile] = running + agg;
                __threadfence();
                *(volatile unsigned*)&st.flag[tile] = 2u;
                sh_prefix = running;
            }
        }
    }
    __syncthreads();
    long long acc = sh_prefix + texcl;
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) {
        const long long x = items[j];
        if (inclusive) {
            acc += x;
            items[j] = acc;
        } else {
            items[j] = acc;
            acc += x;
        }
    }
    tile_store(out, n, base, reverse, sh_tile, items);
}

// ---- float64 reduce-then-scan ------------------------------------------------------
__device__ __forceinline__ double block_sum_f64(double v, double* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (warp == 0) {
        r = lane < nw ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;  // valid in thread 0
}

__global__ void __launch_bounds__(kScanT) scan_f64_tile_sums_kernel(const double* __restrict__ in, int64_t n,
                                                                     bool reverse, double* tile_sums) {
    __shared__ double sh_tile[kScanTile];
    __shared__ double sh[32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    double items[kScanIPT];
    tile_load(in, n, base, reverse, sh_tile, items);
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) t += items[j];
    const double s = block_sum_f64(t, sh);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = s;
}

// One block: exclusive scan of the tile sums in a fixed order, seeded with init.
__global__ void __launch_bounds__(1024) scan_f64_tile_prefix_kernel(double* tile_sums, int64_t ntiles,
                                                                     double init) {
    __shared__ double sh[33];
    const int64_t per = (ntiles + blockDim.x - 1) / blockDim.x;
    const int64_t b = (int64_t)threadIdx.x * per;
    double s = 0.0;
    for (int64_t i = b; i < b + per && i < ntiles; ++i) s += tile_sums[i];
    double total;
    double ex = block_exclusive_scan(s, sh, total);
    double acc = init + ex;
    for (int64_t i = b; i < b + per && i < ntiles; ++i) {
        const double v = tile_sums[i];
        tile_sums[i] = acc;
        acc += v;
    }
}

__global__ void __launch_bounds__(kScanT) scan_f64_downsweep_kernel(const double* __restrict__ in,
                                                                     double* __restrict__ out, int64_t n,
                                                                     bool reverse, bool inclusive,
                                                                     const double* tile_prefix) {
    __shared__ double sh_tile[kScanTile];
    __shared__ double sh[33];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    double items[kScanIPT];
    tile_load(in, n, base, reverse, sh_tile, items);
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) t += items[j];
    double total;
    const double ex = block_exclusive_scan(t, sh, total);
    double acc = tile_prefix[blockIdx.x] + ex;
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) {
        const double x = items[j];
        if (inclusive) {
            acc += x;
            items[j] = acc;
        } else {
            items[j] = acc;
            acc += x;
        }
    }
    tile_store(out, n, base, reverse, sh_tile, items);
}

// ---- segmented reduce: one warp per segment -----------------------------------------
template <class T>
__global__ void __launch_bounds__(256) segreduce_warp_kernel(const int64_t* __restrict__ offsets, int64_t nseg,
                                                             const T* __restrict__ vals, int64_t n_vals, T init,
                                                             T* __restrict__ out, unsigned* err) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    bool bad = false;
    for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nseg; s += warps) {
        const int64_t start = offsets[s], stop = offsets[s + 1];
        T acc = T(0);
        if (start < 0 || stop > n_vals || stop < start) {
            bad = true;
        } else {
            for (int64_t k = start + lane; k < stop; k += 32) acc += vals[k];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) out[s] = init + acc;
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

}  // namespace hyd

using namespace hyd;

namespace hyd {
// Scratch bytes the decoupled look-back needs for n elements.
size_t scan_i64_scratch_bytes(int64_t n) {
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    const size_t flag_bytes = ((size_t)ntiles * 4 + 255) & ~(size_t)255;
    return flag_bytes + 16 * (size_t)ntiles + 256;
}

// int64 scan with caller-provided status scratch (scan_i64_scratch_bytes(n))
// and a 4-byte tile counter; both are reset here on the stream.
int scan_i64_launch_with(const long long* in, long long* out, int64_t n, long long init, bool reverse,
                         bool inclusive, void* status_scratch, unsigned* tile_counter, cudaStream_t stream) {
    if (n == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    const size_t flag_bytes = ((size_t)ntiles * 4 + 255) & ~(size_t)255;
    ScanStatus st;
    st.flag = static_cast<unsigned*>(status_scratch);
    st.aggregate = reinterpret_cast<long long*>(static_cast<unsigned char*>(status_scratch) + flag_bytes);
    st.inclusive = st.aggregate + ntiles;
    st.tile_counter = tile_counter;
    HYD_CUDA_TRY(cudaMemsetAsync(st.flag, 0, (size_t)ntiles * 4, stream));
    HYD_CUDA_TRY(cudaMemsetAsync(st.tile_counter, 0, 4, stream));
    scan_i64_lookback_kernel<<<(unsigned)ntiles, kScanT, 0, stream>>>(in, out, n, init, reverse, inclusive, st,
                                                                       d->d_err);
    return launch_check("scan_i64");
}

// Same, with scratch from the stream's workspace.
int scan_i64_launch(const long long* in, long long* out, int64_t n, long long init, bool reverse,
                    bool inclusive, cudaStream_t stream) {
    if (n == 0) return HYD_CUDA_OK;
    unsigned* counters = nullptr;
    void* scratch = nullptr;
    HYD_TRY(workspace(stream, scan_i64_scratch_bytes(n), &counters, &scratch));
    return scan_i64_launch_with(in, out, n, init, reverse, inclusive, scratch, counters + 8, stream);
}
}  // namespace hyd

extern "C" int hyd_cuda_scan_i64(const int64_t* in, int64_t* out, int64_t n, int64_t init, int reverse,
                                 int inclusive, void* stream) {
    HYD_CHECK_ARG(n >= 0, "scan_i64: negative length");
    HYD_CHECK_ARG(n == 0 || (in != nullptr && out != nullptr), "scan_i64: null buffer");
    HYD_CHECK_ARG(n <= (int64_t)kScanTile * 0x7fffffffLL, "scan_i64: too long");
    return scan_i64_launch(reinterpret_cast<const long long*>(in), reinterpret_cast<long long*>(out), n, init,
                           reverse != 0, inclusive != 0, as_stream(stream));
}

extern "C" int hyd_cuda_scan_f64(const double* in, double* out, int64_t n, double init, int reverse,
                                 int inclusive, void* stream) {
    HYD_CHECK_ARG(n >= 0, "scan_f64: negative length");
    HYD_CHECK_ARG(n == 0 || (in != nullptr && out != nullptr), "scan_f64: null buffer");
    if (n == 0) return HYD_CUDA_OK;
    cudaStream_t s = as_stream(stream);
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    HYD_CHECK_ARG(ntiles <= 0x7fffffffLL, "scan_f64: too long");
    void* scratch = nullptr;
    HYD_TRY(workspace(s, 8 * (size_t)ntiles, nullptr, &scratch));
    double* sums = static_cast<double*>(scratch);
    scan_f64_tile_sums_kernel<<<(unsigned)ntiles, kScanT, 0, s>>>(in, n, reverse != 0, sums);
    scan_f64_tile_prefix_kernel<<<1, 1024, 0, s>>>(sums, ntiles, init);
    scan_f64_downsweep_kernel<<<(unsigned)ntiles, kScanT, 0, s>>>(in, out, n, reverse != 0, inclusive != 0, sums);
    return launch_check("scan_f64");
}

template <class T>
static int segreduce_launch(const int64_t* offsets, int64_t n_offsets, const T* vals, int64_t n_vals, T init,
                            T* out, void* stream, const char* what) {
    HYD_CHECK_ARG(n_offsets >= 1, "%s: need at least one offset", what);
    HYD_CHECK_ARG(offsets != nullptr, "%s: null offsets", what);
    HYD_CHECK_ARG(n_vals >= 0 && (n_vals == 0 || vals != nullptr), "%s: bad values", what);
    const int64_t nseg = n_offsets - 1;
    HYD_CHECK_ARG(nseg == 0 || out != nullptr, "%s: null output", what);
    if (nseg == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    int64_t blocks = (nseg + 7) / 8;
    const int64_t cap = (int64_t)d->sm_count * 8;
    if (blocks > cap) blocks = cap;
    segreduce_warp_kernel<T><<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(offsets, nseg, vals, n_vals, init,
                                                                               out, d->d_err);
    return launch_check(what);
}

extern "C" int hyd_cuda_segmented_reduce_i64(const int64_t* offsets, int64_t n_offsets, const int64_t* vals,
                                             int64_t n_vals, int64_t init, int64_t* out, void* stream) {
    return segreduce_launch<long long>(offsets, n_offsets, reinterpret_cast<const long long*>(vals), n_vals,
                                       (long long)init, reinterpret_cast<long long*>(out), stream,
                                       "segmented_reduce_i64");
}

extern "C" int hyd_cuda_segmented_reduce_f64(const int64_t* offsets, int64_t n_offsets, const double* vals,
                                             int64_t n_vals, double init, double* out, void* stream) {
    return segreduce_launch<double>(offsets, n_offsets, vals, n_vals, init, out, stream, "segmented_reduce_f64");
}
