// hyd_common.cuh -- shared internals of the sm_103a runtime: status/error
// plumbing, the per-device context with per-stream scratch workspaces, and the
// device-side helpers (256-bit streaming loads, counter-based RNG) that every
// kernel file uses.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <unordered_map>

#include "hyd_cuda.h"

namespace hyd {

// ---------------------------------------------------------------- errors ----
int set_error(int status, const char* fmt, ...);
const char* last_error();

#define HYD_CHECK_ARG(cond, ...)                                  \
    do {                                                          \
        if (!(cond)) return ::hyd::set_error(HYD_CUDA_ERR_INVALID, __VA_ARGS__); \
    } while (0)

#define HYD_CUDA_TRY(expr)                                                         \
    do {                                                                           \
        cudaError_t _e = (expr);                                                   \
        if (_e != cudaSuccess)                                                     \
            return ::hyd::set_error(_e == cudaErrorMemoryAllocation ? HYD_CUDA_ERR_NOMEM \
                                                                   : HYD_CUDA_ERR_CUDA, \
                                    "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                                    __FILE__, __LINE__);                            \
    } while (0)

#define HYD_TRY(expr)                 \
    do {                              \
        int _s = (expr);              \
        if (_s != HYD_CUDA_OK) return _s; \
    } while (0)

// Error bits that kernels raise in the per-device error word.
enum : unsigned {
    ERRBIT_BOUNDS = 1u,
    ERRBIT_TIMEOUT = 2u,
};

// ---------------------------------------------------------------- context ---
// Scratch memory for one stream.  The first kCounterBytes hold completion
// counters that kernels leave at zero when they finish; the rest is free-form
// scratch (partials, flags, tiles) that a kernel may use for one launch.
struct Workspace {
    unsigned char* base = nullptr;
    size_t bytes = 0;
};

constexpr size_t kCounterBytes = 4096;

struct Device {
    int id = -1;
    int sm_count = 0;
    int max_smem_optin = 0;
    unsigned* d_err = nullptr;        // error word (device)
    std::mutex mu;
    std::unordered_map<cudaStream_t, Workspace> ws;
    // runtime-owned device buffers (staging for host-pointer entry points)
    std::unordered_map<std::string, Workspace> bufs;
    cudaStream_t side[2] = {nullptr, nullptr};  // pipelining streams
};

// Returns the current device's context, creating it on first use.
int device(Device** out);
// Scratch of at least `bytes` beyond the counter area for `stream`.  Growth
// synchronizes the stream before freeing the old block.
int workspace(cudaStream_t stream, size_t bytes, unsigned** counters, void** scratch);

// Runtime-owned device buffer named `key` of at least `bytes` (grows; the
// caller must not have work in flight on an old block when it grows).
int device_buffer(Device* d, const char* key, size_t bytes, void** p);
// The two non-blocking streams host-pointer entry points pipeline on.
int side_streams(Device* d, cudaStream_t out[2]);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Sets the maximum dynamic shared memory (and, if asked, non-portable cluster
// sizes) for kernel `fn` on device `d`, once per (kernel, device).
int configure_kernel(const void* fn, const Device* d, bool nonportable_cluster);

// Autotuner table lookups (-1 when the shape class was never tuned).
int tune_lookup_stencil(int kind, int64_t h, int64_t w);
int tune_lookup_hist(int64_t bins);

// Kernel launch error check after a <<<>>> launch.
inline int launch_check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(HYD_CUDA_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
    return HYD_CUDA_OK;
}

// ------------------------------------------------------------ device helpers
// SplitMix64 output function over a Weyl sequence indexed by element number
// (Steele, Lea, Flood, OOPSLA 2014); identical to the oracle's generator.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t rand_u64(uint64_t seed_mixed, uint64_t i) {
    return mix64(seed_mixed + (i + 1ULL) * 0x9E3779B97F4A7C15ULL);
}

struct f64x4 { double x, y, z, w; };
struct u64x4 { unsigned long long x, y, z, w; };

// 256-bit read-only streaming loads (sm_100+ `ld.global.nc.v4.b64`), no L1
// allocation: each input byte is read exactly once.
__device__ __forceinline__ f64x4 ldg_stream_f64x4(const double* p) {
    f64x4 r;
    asm volatile("ld.global.nc.L1::no_allocate.v4.f64 {%0,%1,%2,%3}, [%4];"
                 : "=d"(r.x), "=d"(r.y), "=d"(r.z), "=d"(r.w)
                 : "l"(p));
    return r;
}
__device__ __forceinline__ u64x4 ldg_stream_u64x4(const void* p) {
    u64x4 r;
    asm volatile("ld.global.nc.L1::no_allocate.v4.u64 {%0,%1,%2,%3}, [%4];"
                 : "=l"(r.x), "=l"(r.y), "=l"(r.z), "=l"(r.w)
                 : "l"(p));
    return r;
}
__device__ __forceinline__ void stg_f64x4(double* p, f64x4 v) {
    asm volatile("st.global.v4.f64 [%0], {%1,%2,%3,%4};" ::"l"(p), "d"(v.x), "d"(v.y), "d"(v.z),
                 "d"(v.w)
                 : "memory");
}

__device__ __forceinline__ void raise_error(unsigned* err, unsigned bit) { atomicOr(err, bit); }

// Divide/remainder by a runtime-invariant positive int64 divisor with C's
// truncating semantics.  Power-of-two divisors use shifts/masks; others fall
// back to the hardware-emulated 64-bit divide.
struct DivMod64 {
    long long d;
    unsigned long long mask;
    int shift;  // >= 0 when d is a power of two
    __host__ void init(long long dv) {
        d = dv;
        shift = -1;
        mask = 0;
        if (dv > 0 && (dv & (dv - 1)) == 0) {
            int s = 0;
            while ((1LL << s) != dv) ++s;
            shift = s;
            mask = (unsigned long long)dv - 1ULL;
        }
    }
    __device__ __forceinline__ long long rem(long long x) const {
        if (shift >= 0) {
            if (x >= 0) return (long long)((unsigned long long)x & mask);
            // C: the remainder takes the sign of the dividend.
            return -(long long)((0ULL - (unsigned long long)x) & mask);
        }
        return x % d;
    }
};

// ---- mbarrier + bulk asynchronous copies (shared by the TMA kernels) ----------
constexpr unsigned kTmaWaitLimit = 1u << 22;  // polls before a wait gives up

__device__ __forceinline__ void mbar_init(unsigned addr, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned addr, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(addr), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test_wait(unsigned addr, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait (non-blocking polls with a short sleep between them, about a
// quarter of a second in total at the default limit); false when the limit ran
// out.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned addr, unsigned parity,
                                                  unsigned limit = kTmaWaitLimit) {
    for (unsigned it = 0; it < limit; ++it) {
        if (mbar_test_wait(addr, parity)) return true;
        __nanosleep(64);
    }
    return false;
}
// One-dimensional bulk copy global -> shared, completing on an mbarrier.  Both
// addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_load_1d(unsigned dst, const void* src, unsigned bytes, unsigned mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(mbar)
        : "memory");
}

// ---- decoupled look-back: tile status words and the bounded window wait ------
constexpr unsigned kSpinLimit = 1u << 22;  // polls before a look-back gives up

// One tile's status: flag 0 = nothing published, 1 = `bits` hold the tile's
// aggregate, 2 = `bits` hold the inclusive prefix through the tile.  A status
// is written and read as one 16-byte access, so a reader gets a flag together
// with its own value in a single memory round trip and a publisher needs no
// fence between value and flag (the value and flag cannot be seen apart).
struct __align__(16) TileWord {
    unsigned long long flag;
    unsigned long long bits;
};

__device__ __forceinline__ void tile_word_store(TileWord* w, unsigned long long flag, unsigned long long bits) {
    asm volatile("st.volatile.global.v2.u64 [%0], {%1, %2};" ::"l"(w), "l"(flag), "l"(bits) : "memory");
}
__device__ __forceinline__ void tile_word_load(const TileWord* w, unsigned long long& flag,
                                               unsigned long long& bits) {
    asm volatile("ld.volatile.global.v2.u64 {%0, %1}, [%2];" : "=l"(flag), "=l"(bits) : "l"(w) : "memory");
}

template <class T>
__device__ __forceinline__ unsigned long long to_bits(T v) {
    return (unsigned long long)v;
}
template <>
__device__ __forceinline__ unsigned long long to_bits<double>(double v) {
    return (unsigned long long)__double_as_longlong(v);
}
template <class T>
__device__ __forceinline__ T from_bits(unsigned long long b) {
    return (T)b;
}
template <>
__device__ __forceinline__ double from_bits<double>(unsigned long long b) {
    return __longlong_as_double((long long)b);
}

// Warp-wide: lane l watches the status word of tile q = p - l (q < 0: before
// the first tile, reported as flag 2 with bits 0).  Polls until every lane's
// flag is non-zero and returns this lane's flag with its value in `bits`, or
// returns 0 on every lane when `limit` polls went by without that (the caller
// raises ERRBIT_TIMEOUT and abandons the look-back).
__device__ __forceinline__ unsigned lookback_wait_words(const TileWord* words, int64_t p, int lane,
                                                        unsigned long long& bits, unsigned limit = kSpinLimit) {
    const int64_t q = p - lane;
    unsigned long long f = 2ull;
    bits = 0ull;
    if (q >= 0) tile_word_load(&words[q], f, bits);
    unsigned spins = 0;
    while (__any_sync(0xffffffffu, f == 0ull)) {
        if (++spins > limit) return 0u;
        if (f == 0ull) tile_word_load(&words[q], f, bits);
    }
    return (unsigned)f;
}

}  // namespace hyd
