// reduce_rows.cu -- reduction over the last dimension (ND `reduce`).
//
// EReduce (Lowering.hs:723-760) reduces an array of shape [.., n] over its
// trailing axis: for every outer index j, acc = init, then
// acc = f(acc, x[j * n + k]) for k = 0 .. n-1 in order, and out[j] = acc (the
// LoopMapReduction of the C backend).  The reference recognises (+) and (*)
// as reduction operators (CFGCore.hs:236, Redop); these are the ones here.
//   * rows of up to 32 elements: one thread per row, folding in the
//     reference's order -- bit-identical to it, floats included;
//   * longer rows: a warp per row (or a 256-thread block when there are few
//     rows), each lane folding the elements k = lane, lane + W, ... into four
//     interleaved accumulators from the identity, then a fixed tree, then init
//     combined last: deterministic, and within rounding of the serial fold for
//     floats (integers wrap, exact);
//   * a few very long rows: each row split into chunks over many blocks, whose
//     partials a second pass folds in chunk order.
#include <type_traits>

#include "hyd_common.cuh"

namespace hyd {

template <class T, int OP>
__device__ __forceinline__ T rcomb(T a, T b) {
    if constexpr (std::is_integral<T>::value) {
        return OP == HYD_REDOP_ADD ? (T)((unsigned long long)a + (unsigned long long)b)
                                   : (T)((unsigned long long)a * (unsigned long long)b);
    } else {
        return OP == HYD_REDOP_ADD ? __dadd_rn(a, b) : __dmul_rn(a, b);
    }
}
template <class T, int OP>
__device__ __forceinline__ T ridentity() {
    return OP == HYD_REDOP_ADD ? (T)0 : (T)1;
}

template <class T, int OP>
__global__ void rows_serial_kernel(const T* __restrict__ in, int64_t rows, int64_t cols, T init, T* __restrict__ out) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < rows; j += (int64_t)gridDim.x * blockDim.x) {
        T acc = init;
        const T* r = in + j * cols;
        for (int64_t k = 0; k < cols; ++k) acc = rcomb<T, OP>(acc, r[k]);
        out[j] = acc;
    }
}

template <class T, int OP>
__device__ __forceinline__ T warp_tree(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = rcomb<T, OP>(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// this thread's fold of r[k0], r[k0 + W], ... below `end`: four interleaved
// accumulators (loads in flight together), combined in a fixed order
template <class T, int OP, int W>
__device__ __forceinline__ T strided_fold(const T* __restrict__ r, int64_t k0, int64_t end) {
    T a0 = ridentity<T, OP>(), a1 = a0, a2 = a0, a3 = a0;
    int64_t k = k0;
    for (; k + 3 * W < end; k += 4 * W) {
        a0 = rcomb<T, OP>(a0, __ldg(r + k));
        a1 = rcomb<T, OP>(a1, __ldg(r + k + W));
        a2 = rcomb<T, OP>(a2, __ldg(r + k + 2 * W));
        a3 = rcomb<T, OP>(a3, __ldg(r + k + 3 * W));
    }
    for (; k < end; k += W) a0 = rcomb<T, OP>(a0, __ldg(r + k));
    return rcomb<T, OP>(rcomb<T, OP>(a0, a1), rcomb<T, OP>(a2, a3));
}

template <class T, int OP>
__global__ void rows_warp_kernel(const T* __restrict__ in, int64_t rows, int64_t cols, T init, T* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t j = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < rows; j += warps) {
        T acc = warp_tree<T, OP>(strided_fold<T, OP, 32>(in + j * cols, lane, cols));
        if (lane == 0) out[j] = rcomb<T, OP>(init, acc);
    }
}

// Block j % nchunks of row j / nchunks folds its chunk [c * chunk, ..) of
// the row into part[j] (nchunks == 1: the whole row, then init, into out).
template <class T, int OP>
__global__ void __launch_bounds__(256) rows_block_kernel(const T* __restrict__ in, int64_t rows, int64_t cols,
                                                         int64_t nchunks, int64_t chunk, T init, T* __restrict__ out,
                                                         T* __restrict__ part) {
    __shared__ T wpart[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t j = blockIdx.x; j < rows * nchunks; j += gridDim.x) {
        const int64_t row = j / nchunks, c = j % nchunks;
        const int64_t lo = c * chunk, hi = lo + chunk < cols ? lo + chunk : cols;
        T acc = warp_tree<T, OP>(strided_fold<T, OP, 256>(in + row * cols, lo + threadIdx.x, hi));
        if (lane == 0) wpart[warp] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            T t = wpart[0];
            for (int w = 1; w < 8; ++w) t = rcomb<T, OP>(t, wpart[w]);
            if (nchunks == 1) out[row] = rcomb<T, OP>(init, t);
            else part[j] = t;
        }
        __syncthreads();
    }
}

// init, then the chunks' partials of each row in chunk order
template <class T, int OP>
__global__ void rows_combine_kernel(const T* __restrict__ part, int64_t rows, int64_t nchunks, T init,
                                    T* __restrict__ out) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < rows; j += (int64_t)gridDim.x * blockDim.x) {
        T acc = init;
        for (int64_t c = 0; c < nchunks; ++c) acc = rcomb<T, OP>(acc, part[j * nchunks + c]);
        out[j] = acc;
    }
}

template <class T, int OP>
static int launch_rows(const T* in, int64_t rows, int64_t cols, T init, T* out, cudaStream_t s) {
    Device* d = nullptr;
    HYD_TRY(device(&d));
    const int64_t cap = (int64_t)d->sm_count * 8;
    if (cols <= 32) {
        const int64_t want = (rows + 255) / 256;
        rows_serial_kernel<T, OP><<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(in, rows, cols, init, out);
    } else if (rows >= (int64_t)d->sm_count * 16) {
        const int64_t want = (rows + 7) / 8;
        rows_warp_kernel<T, OP><<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(in, rows, cols, init, out);
    } else {
        // enough blocks for the whole GPU: long rows split into chunks of at
        // least 2^14 elements
        int64_t nchunks = 1, chunk = cols;
        const int64_t want_blocks = (int64_t)d->sm_count * 8;
        if (rows < want_blocks && cols >= (int64_t)1 << 15) {
            nchunks = (want_blocks + rows - 1) / rows;
            const int64_t most = (cols + ((int64_t)1 << 14) - 1) >> 14;
            if (nchunks > most) nchunks = most;
            chunk = (cols + nchunks - 1) / nchunks;
            nchunks = (cols + chunk - 1) / chunk;
        }
        T* part = nullptr;
        if (nchunks > 1) {
            unsigned* counters = nullptr;
            void* scratch = nullptr;
            HYD_TRY(workspace(s, (size_t)(rows * nchunks) * sizeof(T), &counters, &scratch));
            part = static_cast<T*>(scratch);
        }
        const int64_t blocks = rows * nchunks;
        rows_block_kernel<T, OP><<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(in, rows, cols, nchunks,
                                                                                         chunk, init, out, part);
        if (nchunks > 1) {
            HYD_TRY(launch_check("reduce_rows"));
            rows_combine_kernel<T, OP><<<1, 256, 0, s>>>(part, rows, nchunks, init, out);
        }
    }
    return launch_check("reduce_rows");
}

template <class T>
static int reduce_rows(const T* in, int64_t rows, int64_t cols, int op, T init, T* out, void* stream,
                       const char* what) {
    HYD_CHECK_ARG(rows >= 0 && cols >= 0, "%s: negative shape", what);
    HYD_CHECK_ARG(op == HYD_REDOP_ADD || op == HYD_REDOP_MUL, "%s: unknown operator %d", what, op);
    HYD_CHECK_ARG(rows == 0 || out != nullptr, "%s: null output", what);
    HYD_CHECK_ARG(rows * cols == 0 || in != nullptr, "%s: null input", what);
    if (rows == 0) return HYD_CUDA_OK;
    cudaStream_t s = as_stream(stream);
    return op == HYD_REDOP_ADD ? launch_rows<T, HYD_REDOP_ADD>(in, rows, cols, init, out, s)
                               : launch_rows<T, HYD_REDOP_MUL>(in, rows, cols, init, out, s);
}

}  // namespace hyd

using namespace hyd;

extern "C" int hyd_cuda_reduce_rows_i64(const int64_t* in, int64_t rows, int64_t cols, int op, int64_t init,
                                        int64_t* out, void* stream) {
    return reduce_rows<int64_t>(in, rows, cols, op, init, out, stream, "reduce_rows_i64");
}

extern "C" int hyd_cuda_reduce_rows_f64(const double* in, int64_t rows, int64_t cols, int op, double init, double* out,
                                        void* stream) {
    return reduce_rows<double>(in, rows, cols, op, init, out, stream, "reduce_rows_f64");
}
