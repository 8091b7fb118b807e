// sort.cu -- sort_indices (stable LSD radix, 8-bit digits) and gather.
//
// Replaces the runtime's serial hyd_radix_sort_entries / hyd_sort_indices
// (runtime/hydrangea_runtime.h:386-456), reached from `sort_indices`
// (Lowering.hs:961-965).  The result must be the same permutation, so the
// digit function and pass count are the runtime's: digit p of a key is
// (key >> 8p) & 0xFF on the signed key, and the number of passes is the
// number of bytes of max(0, max key) (at least one).  Any stable LSD sort with
// those digits yields exactly that permutation.
//
// Per pass, three launches over tiles of 4096 elements:
//  1. digit histogram per tile (shared-memory u32 atomics), written
//     digit-major so that
//  2. one exclusive scan (the decoupled look-back int64 scan) turns the counts
//     into each (digit, tile)'s first output position, and
//  3. a stable scatter: each warp ranks its 256 contiguous elements in 8 rounds
//     of 32 among the lanes holding the same digit (one ballot per digit bit;
//     lanes in element order, running counts per (warp, digit) in shared
//     memory), so equal digits keep input order.
// Keys travel with their original index; the first pass generates the
// indices, the last pass writes only the permutation.
#include "hyd_common.cuh"

namespace hyd {

size_t scan_i64_scratch_bytes(int64_t n);
int scan_i64_launch_with(const long long* in, long long* out, int64_t n, long long init, bool reverse,
                         bool inclusive, void* status_scratch, unsigned* tile_counter, cudaStream_t stream);

constexpr int kSortT = 512;
constexpr int kSortWarps = kSortT / 32;
constexpr int kSortIPW = 256;                    // elements per warp per tile
constexpr int kSortTile = kSortWarps * kSortIPW;  // 4096

__device__ __forceinline__ unsigned digit_of(long long key, int shift) {
    return (unsigned)((key >> shift) & 0xFF);
}

__global__ void __launch_bounds__(kSortT) radix_hist_kernel(const long long* __restrict__ keys, int64_t n,
                                                             int shift, long long* __restrict__ counts,
                                                             int64_t ntiles) {
    __shared__ unsigned h[256];
    for (int i = threadIdx.x; i < 256; i += kSortT) h[i] = 0u;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += kSortT) {
        const int64_t e = base + i;
        if (e < n) atomicAdd(&h[digit_of(keys[e], shift)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += kSortT) counts[(int64_t)d * ntiles + blockIdx.x] = h[d];
}

// kFirst: values are the element indices (not read); kLast: keys are not written.
template <bool kFirst, bool kLast>
__global__ void __launch_bounds__(kSortT) radix_scatter_kernel(const long long* __restrict__ keys_in,
                                                                const long long* __restrict__ vals_in,
                                                                long long* __restrict__ keys_out,
                                                                long long* __restrict__ vals_out, int64_t n,
                                                                int shift, const long long* __restrict__ offsets,
                                                                int64_t ntiles) {
    __shared__ unsigned wcount[kSortWarps][256];
    __shared__ long long tile_off[256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortT) (&wcount[0][0])[i] = 0u;
    for (int d = threadIdx.x; d < 256; d += kSortT) tile_off[d] = offsets[(int64_t)d * ntiles + blockIdx.x];
    __syncthreads();
    const int64_t wbase = (int64_t)blockIdx.x * kSortTile + (int64_t)warp * kSortIPW;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    constexpr int R = kSortIPW / 32;
    long long k[R], v[R];
    unsigned dig[R], rank[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int64_t e = wbase + r * 32 + lane;
        const bool ok = e < n;
        k[r] = ok ? keys_in[e] : 0;
        v[r] = ok ? (kFirst ? (long long)e : vals_in[e]) : 0;
        dig[r] = ok ? digit_of(k[r], shift) : 0x100u;  // 0x100: past the end
        // the lanes holding the same digit: one ballot per digit bit (the ALU
        // pipe) rather than a match instruction (the ADU pipe, which binds)
        unsigned peers = __ballot_sync(0xffffffffu, ok);
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            const unsigned bb = __ballot_sync(0xffffffffu, (dig[r] >> b) & 1u);
            peers &= ((dig[r] >> b) & 1u) ? bb : ~bb;
        }
        unsigned prior = 0;
        if (ok) prior = wcount[warp][dig[r]];
        __syncwarp();
        rank[r] = prior + __popc(peers & lt);
        if (ok && (peers & lt) == 0u) wcount[warp][dig[r]] = prior + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // exclusive prefix over warps for each digit (warp order = element order)
    for (int d = threadIdx.x; d < 256; d += kSortT) {
        unsigned run = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            const unsigned c = wcount[w][d];
            wcount[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (dig[r] < 256u) {
            const int64_t pos = tile_off[dig[r]] + wcount[warp][dig[r]] + rank[r];
            if (!kLast) keys_out[pos] = k[r];
            vals_out[pos] = v[r];
        }
    }
}

__global__ void max_key_kernel(const long long* __restrict__ keys, int64_t n, unsigned long long* out) {
    long long m = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = keys[i] > m ? keys[i] : m;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long y = __shfl_xor_sync(0xffffffffu, m, o);
        m = y > m ? y : m;
    }
    if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(out, (unsigned long long)m);
}

template <class T>
__global__ void gather_kernel(const long long* __restrict__ perm, int64_t n, const T* __restrict__ src,
                              int64_t src_n, T* __restrict__ out, unsigned* err) {
    bool bad = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const long long p = perm[i];
        if ((unsigned long long)p < (unsigned long long)src_n) out[i] = src[p];
        else bad = true;
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// Sort with a known number of 8-bit passes.  Scratch from the stream workspace.
int sort_indices_passes(const long long* keys, int64_t n, int passes, long long* perm, cudaStream_t stream) {
    const int64_t ntiles = (n + kSortTile - 1) / kSortTile;
    void* scratch = nullptr;
    unsigned* counters = nullptr;
    const size_t cnt_bytes = ((size_t)256 * ntiles * 8 + 255) & ~(size_t)255;
    const size_t buf_bytes = ((size_t)n * 8 + 255) & ~(size_t)255;
    const size_t scan_bytes = (scan_i64_scratch_bytes(256 * ntiles) + 255) & ~(size_t)255;
    HYD_TRY(workspace(stream, 2 * cnt_bytes + 3 * buf_bytes + scan_bytes, &counters, &scratch));
    unsigned char* s = static_cast<unsigned char*>(scratch);
    void* scan_scratch = s + 2 * cnt_bytes + 3 * buf_bytes;
    long long* counts = reinterpret_cast<long long*>(s);
    long long* offsets = reinterpret_cast<long long*>(s + cnt_bytes);
    long long* kb[2] = {reinterpret_cast<long long*>(s + 2 * cnt_bytes),
                        reinterpret_cast<long long*>(s + 2 * cnt_bytes + buf_bytes)};
    long long* vb = reinterpret_cast<long long*>(s + 2 * cnt_bytes + 2 * buf_bytes);
    // value ping-pong: vb <-> perm, arranged so the last pass lands in perm
    long long* vbufs[2];
    vbufs[(passes - 1) & 1] = perm;
    vbufs[passes & 1] = vb;
    const long long* kin = keys;
    const long long* vin = nullptr;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        radix_hist_kernel<<<(unsigned)ntiles, kSortT, 0, stream>>>(kin, n, shift, counts, ntiles);
        HYD_TRY(launch_check("radix_hist"));
        HYD_TRY(scan_i64_launch_with(counts, offsets, 256 * ntiles, 0, false, false, scan_scratch, counters + 8,
                                     stream));
        long long* kout = kb[p & 1];
        long long* vout = vbufs[p & 1];
        const bool first = p == 0, last = p == passes - 1;
        dim3 g((unsigned)ntiles);
        if (first && last)
            radix_scatter_kernel<true, true><<<g, kSortT, 0, stream>>>(kin, vin, kout, vout, n, shift, offsets, ntiles);
        else if (first)
            radix_scatter_kernel<true, false><<<g, kSortT, 0, stream>>>(kin, vin, kout, vout, n, shift, offsets, ntiles);
        else if (last)
            radix_scatter_kernel<false, true><<<g, kSortT, 0, stream>>>(kin, vin, kout, vout, n, shift, offsets, ntiles);
        else
            radix_scatter_kernel<false, false><<<g, kSortT, 0, stream>>>(kin, vin, kout, vout, n, shift, offsets, ntiles);
        HYD_TRY(launch_check("radix_scatter"));
        kin = kout;
        vin = vout;
    }
    return HYD_CUDA_OK;
}

}  // namespace hyd

using namespace hyd;

extern "C" int hyd_cuda_sort_indices_i64(const int64_t* keys, int64_t n, int64_t* perm, void* stream) {
    HYD_CHECK_ARG(n >= 0, "sort_indices: negative length");
    HYD_CHECK_ARG(n == 0 || (keys != nullptr && perm != nullptr), "sort_indices: null buffer");
    HYD_CHECK_ARG(n < (1LL << 40), "sort_indices: too long");
    if (n == 0) return HYD_CUDA_OK;
    cudaStream_t s = as_stream(stream);
    Device* d = nullptr;
    HYD_TRY(device(&d));
    unsigned* counters = nullptr;
    HYD_TRY(workspace(s, 0, &counters, nullptr));
    unsigned long long* dmax = reinterpret_cast<unsigned long long*>(counters + 16);
    HYD_CUDA_TRY(cudaMemsetAsync(dmax, 0, 8, s));
    int64_t blocks = (n + 255) / 256;
    if (blocks > d->sm_count * 4) blocks = d->sm_count * 4;
    max_key_kernel<<<(unsigned)blocks, 256, 0, s>>>(reinterpret_cast<const long long*>(keys), n, dmax);
    HYD_TRY(launch_check("sort_indices max key"));
    unsigned long long mk = 0;
    HYD_CUDA_TRY(cudaMemcpyAsync(&mk, dmax, 8, cudaMemcpyDeviceToHost, s));
    HYD_CUDA_TRY(cudaStreamSynchronize(s));
    int passes = 0;
    for (unsigned long long m = mk; m; m >>= 8) ++passes;
    if (passes == 0) passes = 1;
    return sort_indices_passes(reinterpret_cast<const long long*>(keys), n, passes,
                               reinterpret_cast<long long*>(perm), s);
}

extern "C" int hyd_cuda_sort_indices_bits_i64(const int64_t* keys, int64_t n, int key_bits, int64_t* perm,
                                              void* stream) {
    HYD_CHECK_ARG(n >= 0, "sort_indices_bits: negative length");
    HYD_CHECK_ARG(key_bits >= 0 && key_bits <= 64, "sort_indices_bits: key_bits in [0, 64]");
    HYD_CHECK_ARG(n == 0 || (keys != nullptr && perm != nullptr), "sort_indices_bits: null buffer");
    if (n == 0) return HYD_CUDA_OK;
    int passes = (key_bits + 7) / 8;
    if (passes == 0) passes = 1;
    return sort_indices_passes(reinterpret_cast<const long long*>(keys), n, passes,
                               reinterpret_cast<long long*>(perm), as_stream(stream));
}

template <class T>
static int gather_launch(const int64_t* perm, int64_t n, const T* src, int64_t src_n, T* out, void* stream) {
    HYD_CHECK_ARG(n >= 0 && src_n >= 0, "gather: negative length");
    HYD_CHECK_ARG(n == 0 || (perm && src && out), "gather: null buffer");
    if (n == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    int64_t blocks = (n + 255) / 256;
    if (blocks > d->sm_count * 8) blocks = d->sm_count * 8;
    gather_kernel<T><<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(reinterpret_cast<const long long*>(perm), n,
                                                                      src, src_n, out, d->d_err);
    return launch_check("gather");
}

extern "C" int hyd_cuda_gather_i64(const int64_t* perm, int64_t n, const int64_t* src, int64_t src_n, int64_t* out,
                                   void* stream) {
    return gather_launch<long long>(perm, n, reinterpret_cast<const long long*>(src), src_n,
                                    reinterpret_cast<long long*>(out), stream);
}

extern "C" int hyd_cuda_gather_f64(const int64_t* perm, int64_t n, const double* src, int64_t src_n, double* out,
                                   void* stream) {
    return gather_launch<double>(perm, n, src, src_n, out, stream);
}

extern "C" int hyd_cuda_gather_i32(const int64_t* perm, int64_t n, const int32_t* src, int64_t src_n, int32_t* out,
                                   void* stream) {
    return gather_launch<int>(perm, n, reinterpret_cast<const int*>(src), src_n, reinterpret_cast<int*>(out), stream);
}
