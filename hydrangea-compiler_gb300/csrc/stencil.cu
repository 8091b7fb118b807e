// stencil.cu -- 2-D clamp stencils with the 5-point footprint, and `iterate`
// over them.
//
// Replaces the split-region stencil loops of the reference
// (Lowering.hs:2562-2661 interior + clamped boundary strips, each an
// `omp parallel for`) and the ping-pong `iterate` of Lowering.hs:840-858 /
// CFGOpt.hs:795-810.  Per point the body is the program text evaluated left
// to right (a = acc (-1) 0, b = acc 1 0, c = acc 0 (-1), d = acc 0 1,
// e = acc 0 0):
//   LAPLACIAN     a + b + c + d + (e * -4.0)          (bench/stencil/stencil_2d.hyd)
//   JACOBI        (a + b + c + d) / 4.0                (bench/stencil/jacobi_2d.hyd)
//   HEAT          e + 0.1 * (a + b + c + d - 4.0 * e)  (the 8192^2 heat step)
//   HEAT_EXAMPLE  (a + b + c + d + e) / 5.0            (examples/heat_2d.hyd)
// Results are bit-identical to the C backend: no contraction except where it
// is exact -- `t3 - 4e` and `t3 + e*-4` are one fma because 4e is exact (for
// |e| < DBL_MAX/4), and /4.0 is *0.25 (both correctly rounded, same value).
//
// GB300 design.  fp64 runs at ~1.9 DFMA/clk/SM on this part, so a 5-point fp64
// step is bound by the FP64 pipe (6 DP ops per point for HEAT), not by HBM.
// The kernel therefore spends nothing but DP ops in its inner loop:
//  * a persistent grid walks 16 x 128 output tiles; each tile plus its halo
//    (rows -1..+1, columns -2..+2 so the TMA x coordinate stays 16-byte
//    aligned) is brought into shared memory by a 2-D TMA load
//    (cp.async.bulk.tensor) completing on an mbarrier, double-buffered so the
//    next tile streams in while this one computes; out-of-range rows/columns
//    are zero-filled by TMA and never read (clamp maps inside the grid);
//  * each thread owns one column of 8 rows with a sliding vertical window
//    (3 shared loads per point), interior tiles skip all clamp arithmetic;
//  * every mbarrier wait is bounded: on timeout the kernel raises an error bit
//    and returns instead of hanging.
// `iterate` runs as a captured CUDA graph of the step launches (ping-pong
// buffers, one tensor map per buffer), cached per (kind, shape, buffers,
// steps).  Shapes TMA cannot describe (odd width, misaligned base) use a
// plain clamped kernel with the same arithmetic.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <map>
#include <tuple>

#include "fp64_emu.cuh"
#include "hyd_common.cuh"

namespace hyd {

enum { ST_LAPLACIAN = 0, ST_JACOBI = 1, ST_HEAT = 2, ST_HEAT_EXAMPLE = 3 };

// EMU: how many of the three additions a + b, + c, + d run on the integer
// pipe (dadd_pos, bit-identical to __dadd_rn); the rest use the FP64 unit.
template <int KIND, int EMU>
__device__ __forceinline__ double stencil_body(double a, double b, double c, double d, double e) {
    const double t1 = EMU >= 1 ? dadd_pos(a, b) : __dadd_rn(a, b);
    const double t2 = EMU >= 2 ? dadd_pos(t1, c) : __dadd_rn(t1, c);
    const double t3 = EMU >= 3 ? dadd_pos(t2, d) : __dadd_rn(t2, d);
    if (KIND == ST_LAPLACIAN) return __fma_rn(e, -4.0, t3);
    if (KIND == ST_JACOBI) return __dmul_rn(t3, 0.25);
    if (KIND == ST_HEAT) {
        const double lap = __fma_rn(-4.0, e, t3);
        return __dadd_rn(e, __dmul_rn(0.1, lap));
    }
    return ddiv_small_rn<5>(__dadd_rn(t3, e));  // = __ddiv_rn(., 5.0), bit for bit
}

// ---------------------------------------------------------------- plain path
template <int KIND, int EMU>
__global__ void __launch_bounds__(256) stencil_plain_kernel(const double* __restrict__ in,
                                                            double* __restrict__ out, int64_t h,
                                                            int64_t w) {
    const int64_t j = (int64_t)blockIdx.x * 32 + (threadIdx.x & 31);
    const int64_t i = (int64_t)blockIdx.y * 8 + (threadIdx.x >> 5);
    if (i >= h || j >= w) return;
    const int64_t im = i > 0 ? i - 1 : 0, ip = i + 1 < h ? i + 1 : h - 1;
    const int64_t jm = j > 0 ? j - 1 : 0, jp = j + 1 < w ? j + 1 : w - 1;
    out[i * w + j] = stencil_body<KIND, EMU>(in[im * w + j], in[ip * w + j], in[i * w + jm],
                                        in[i * w + jp], in[i * w + j]);
}

// ---------------------------------------------------------------- TMA path
// Tile shapes: TH output rows x TW output columns, 256 threads, TW in {32, 64,
// 128} so that a thread owns one column of TH*TW/256 consecutive rows.  The
// input box adds a 1-row halo above/below and a 2-column halo left/right (the
// TMA x coordinate must stay 16-byte aligned).
constexpr int kStThreads = 256;

template <int TH, int TW>
struct TileShape {
    static constexpr int kBoxW = TW + 4;
    static constexpr int kBoxH = TH + 2;
    static constexpr int kRowsPerThread = TH * TW / kStThreads;
    static constexpr int kStageBytes = kBoxW * kBoxH * 8;
    static constexpr int kStageStride = (kStageBytes + 1023) & ~1023;
    static constexpr size_t kSmem = 2 * (size_t)kStageStride + 64 + 1024;
    static_assert(TW == 32 || TW == 64 || TW == 128, "TW must divide the thread count");
    static_assert(TH * TW % kStThreads == 0 && kRowsPerThread >= 1, "tile must cover the threads");
    static_assert(kBoxW <= 256 && kBoxH <= 256, "TMA box limit");
};

__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap* map, int x, int y,
                                            unsigned mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}

template <int KIND, int kTH, int kTW, int EMU>
__global__ void __launch_bounds__(kStThreads)
    stencil_tma_kernel(const __grid_constant__ CUtensorMap in_map, double* __restrict__ out,
                       int h, int w, unsigned* err) {
    using S = TileShape<kTH, kTW>;
    constexpr int kBoxW = S::kBoxW;
    constexpr int kStageBytes = S::kStageBytes;
    constexpr int kStageStride = S::kStageStride;
    constexpr int kRowsPerThread = S::kRowsPerThread;
    extern __shared__ __align__(1024) unsigned char sm_raw[];
    // stages at 1024-byte aligned offsets, barriers after them
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(sm_raw) + 1023) & ~uintptr_t(1023));
    // stage s at base + s*kStageStride, its barrier at bars + 8*s
    const unsigned stage0 = (unsigned)__cvta_generic_to_shared(base);
    const unsigned bar0 = stage0 + 2 * kStageStride;
    const int ntj = (w + kTW - 1) / kTW;
    const int nti = (h + kTH - 1) / kTH;
    const int ntiles = nti * ntj;
    if (threadIdx.x == 0) {
        mbar_init(bar0, 1);
        mbar_init(bar0 + 8, 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();

    int tile = blockIdx.x;
    if (threadIdx.x == 0 && tile < ntiles) {
        mbar_expect_tx(bar0, kStageBytes);
        tma_load_2d(stage0, &in_map, (tile % ntj) * kTW - 2, (tile / ntj) * kTH - 1, bar0);
    }
    const int col = threadIdx.x % kTW;
    const int rgrp = threadIdx.x / kTW;  // 0..1: rows rgrp*8 .. rgrp*8+7
    bool timed_out = false;
    int it = 0;
    for (; tile < ntiles; ++it, tile += gridDim.x) {
        const int s = it & 1;
        const unsigned parity = (unsigned)(it >> 1) & 1u;  // use count of stage s, mod 2
        const int next = tile + gridDim.x;
        if (threadIdx.x == 0 && next < ntiles) {
            const unsigned so = (unsigned)(s ^ 1);
            mbar_expect_tx(bar0 + 8 * so, kStageBytes);
            tma_load_2d(stage0 + so * kStageStride, &in_map, (next % ntj) * kTW - 2, (next / ntj) * kTH - 1,
                        bar0 + 8 * so);
        }
        const bool ok = mbar_wait_bounded(bar0 + 8 * (unsigned)s, parity);
        if (__syncthreads_or(!ok)) {  // block-uniform decision
            timed_out = true;
            break;
        }
        const double* sm = reinterpret_cast<const double*>(base + s * kStageStride);
        const int i0 = (tile / ntj) * kTH, j0 = (tile % ntj) * kTW;
        const int j = j0 + col;
        const bool interior = i0 >= 1 && i0 + kTH + 1 <= h && j0 >= 1 && j0 + kTW + 1 <= w;
        const int r0 = rgrp * kRowsPerThread;
        if (interior) {
            // smem row r <-> global row i0 - 1 + r; smem col c <-> global col j0 - 2 + c
            const int c = col + 2;
            double up = sm[(r0) * kBoxW + c];
            double mid = sm[(r0 + 1) * kBoxW + c];
            double* o = out + (int64_t)(i0 + r0) * w + j;
#pragma unroll
            for (int k = 0; k < kRowsPerThread; ++k) {
                const int r = r0 + 1 + k;
                const double dn = sm[(r + 1) * kBoxW + c];
                const double lf = sm[r * kBoxW + c - 1];
                const double rt = sm[r * kBoxW + c + 1];
                o[(int64_t)k * w] = stencil_body<KIND, EMU>(up, dn, lf, rt, mid);
                up = mid;
                mid = dn;
            }
        } else if (j < w) {
            const int jm = (j > 0 ? j - 1 : 0) - j0 + 2, jp = (j + 1 < w ? j + 1 : w - 1) - j0 + 2;
            const int jc = col + 2;
#pragma unroll
            for (int k = 0; k < kRowsPerThread; ++k) {
                const int i = i0 + r0 + k;
                if (i < h) {
                    const int im = (i > 0 ? i - 1 : 0) - i0 + 1, ip = (i + 1 < h ? i + 1 : h - 1) - i0 + 1;
                    const int ic = i - i0 + 1;
                    out[(int64_t)i * w + j] = stencil_body<KIND, EMU>(sm[im * kBoxW + jc], sm[ip * kBoxW + jc],
                                                                 sm[ic * kBoxW + jm], sm[ic * kBoxW + jp],
                                                                 sm[ic * kBoxW + jc]);
                }
            }
        }
        __syncthreads();  // stage s fully read before it is refilled next iteration
    }
    if (timed_out) {
        if (threadIdx.x == 0) raise_error(err, ERRBIT_TIMEOUT);
        // wait (bounded) for the copies that may still land in this CTA's
        // stages: the stage being waited on and the one prefetched after it
        mbar_wait_bounded(bar0 + 8 * (unsigned)(it & 1), (unsigned)(it >> 1) & 1u);
        if (tile + (int)gridDim.x < ntiles)
            mbar_wait_bounded(bar0 + 8 * (unsigned)((it + 1) & 1), (unsigned)((it + 1) >> 1) & 1u);
    }
}


// --- driver entry point for tensor-map encoding --------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
    }
    return fn;
}

static bool tma_ok(const double* p, int64_t h, int64_t w) {
    return encode_fn() != nullptr && (reinterpret_cast<uintptr_t>(p) & 15) == 0 && (w % 2) == 0 &&
           w >= 2 && h >= 1 && w <= (1LL << 31) - 1 && h <= (1LL << 31) - 1;
}

static int make_map(CUtensorMap* map, const double* p, int64_t h, int64_t w, int box_w, int box_h) {
    cuuint64_t dims[2] = {(cuuint64_t)w, (cuuint64_t)h};
    cuuint64_t strides[1] = {(cuuint64_t)w * 8};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(p), dims, strides, box,
                             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(HYD_CUDA_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return HYD_CUDA_OK;
}

// Variants (index = the autotuner's choice) = shape + kShapes * level.
// Shapes: 0 is the reference's fixed 32 x 32 polyhedral tile
// (Polyhedral.hs:196-204), 1-5 GPU-shaped TMA tiles, 6 the plain kernel.
// Levels: how many of the three sum additions run on the integer pipe
// (kEmuLevels[level]); every variant gives bit-identical results.
struct TileVariant {
    int th, tw;
};
static const TileVariant kTiles[] = {{32, 32}, {16, 128}, {16, 64}, {32, 64}, {8, 128}, {32, 128}};
constexpr int kNumTiles = sizeof(kTiles) / sizeof(kTiles[0]);
constexpr int kShapes = kNumTiles + 1;     // + the plain (non-TMA) kernel
constexpr int kPlainShape = kNumTiles;
constexpr int kEmuLevels[] = {0, 2, 3};
constexpr int kNumLevels = sizeof(kEmuLevels) / sizeof(kEmuLevels[0]);
constexpr int kNumVariants = kShapes * kNumLevels;
constexpr int kDefaultVariant = kPlainShape + kShapes;  // plain kernel, 2 integer-pipe sums
                                                        // (fastest at 8192^2 heat on GB300)

template <int KIND, int TH, int TW, int EMU>
static int launch_tma(const CUtensorMap* map, double* out, int64_t h, int64_t w, const Device* d, cudaStream_t stream) {
    using S = TileShape<TH, TW>;
    auto k = stencil_tma_kernel<KIND, TH, TW, EMU>;
    HYD_TRY(configure_kernel((const void*)k, d, false));
    const int64_t ntiles = ((h + TH - 1) / TH) * ((w + TW - 1) / TW);
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kStThreads, S::kSmem);
    if (occ < 1) occ = 1;
    int64_t grid = (int64_t)d->sm_count * occ;
    if (grid > ntiles) grid = ntiles;
    k<<<(unsigned)grid, kStThreads, S::kSmem, stream>>>(*map, out, (int)h, (int)w, d->d_err);
    return HYD_CUDA_OK;
}

template <int KIND, int EMU>
static int launch_shape(const CUtensorMap* map, const double* in, double* out, int64_t h, int64_t w, int shape,
                        const Device* d, cudaStream_t stream) {
    switch (shape) {
        case 0: HYD_TRY((launch_tma<KIND, 32, 32, EMU>(map, out, h, w, d, stream))); break;
        case 1: HYD_TRY((launch_tma<KIND, 16, 128, EMU>(map, out, h, w, d, stream))); break;
        case 2: HYD_TRY((launch_tma<KIND, 16, 64, EMU>(map, out, h, w, d, stream))); break;
        case 3: HYD_TRY((launch_tma<KIND, 32, 64, EMU>(map, out, h, w, d, stream))); break;
        case 4: HYD_TRY((launch_tma<KIND, 8, 128, EMU>(map, out, h, w, d, stream))); break;
        case 5: HYD_TRY((launch_tma<KIND, 32, 128, EMU>(map, out, h, w, d, stream))); break;
        default: {
            dim3 grid((unsigned)((w + 31) / 32), (unsigned)((h + 7) / 8));
            stencil_plain_kernel<KIND, EMU><<<grid, 256, 0, stream>>>(in, out, h, w);
        }
    }
    return launch_check("stencil2d_f64");
}

template <int KIND>
static int launch_step_kind(const CUtensorMap* map, const double* in, double* out, int64_t h, int64_t w,
                            int variant, const Device* d, cudaStream_t stream) {
    const int shape = variant % kShapes;
    switch (kEmuLevels[variant / kShapes]) {
        case 2: return launch_shape<KIND, 2>(map, in, out, h, w, shape, d, stream);
        case 3: return launch_shape<KIND, 3>(map, in, out, h, w, shape, d, stream);
        default: return launch_shape<KIND, 0>(map, in, out, h, w, shape, d, stream);
    }
}

static int launch_step(int kind, const CUtensorMap* map, const double* in, double* out, int64_t h, int64_t w,
                       int variant, const Device* d, cudaStream_t stream) {
    switch (kind) {
        case ST_LAPLACIAN: return launch_step_kind<ST_LAPLACIAN>(map, in, out, h, w, variant, d, stream);
        case ST_JACOBI: return launch_step_kind<ST_JACOBI>(map, in, out, h, w, variant, d, stream);
        case ST_HEAT: return launch_step_kind<ST_HEAT>(map, in, out, h, w, variant, d, stream);
        default: return launch_step_kind<ST_HEAT_EXAMPLE>(map, in, out, h, w, variant, d, stream);
    }
}

// Variant for (kind, h, w): the autotuner's cached choice, else the default;
// shapes TMA cannot describe always take the plain kernel.
static int choose_variant(int kind, const double* a, const double* b, int64_t h, int64_t w, int forced) {
    int v = kDefaultVariant;
    if (forced >= 0 && forced < kNumVariants) {
        v = forced;
    } else {
        const int t = tune_lookup_stencil(kind, h, w);
        if (t >= 0 && t < kNumVariants) v = t;
    }
    const bool tma = tma_ok(a, h, w) && (b == nullptr || tma_ok(b, h, w));
    if (!tma) v = (v / kShapes) * kShapes + kPlainShape;  // same level, plain kernel
    return v;
}

static int maps_for(int variant, const double* p, int64_t h, int64_t w, CUtensorMap* map) {
    const int shape = variant % kShapes;
    if (shape >= kNumTiles) return HYD_CUDA_OK;
    return make_map(map, p, h, w, kTiles[shape].tw + 4, kTiles[shape].th + 2);
}

// ---- other boundary conditions -----------------------------------------------
// `stencil wrap`, `stencil mirror` and `stencil (constant c)` (Syntax.hs:416-426)
// with the same 5-point kinds and arithmetic.  Per dimension the neighbour index
// is the one genBnd1DVar computes (Lowering.hs:2762-2812); for the footprint's
// offsets of +-1 its formulas reduce to
//   wrap    -1 -> n - 1,  n -> 0;
//   mirror  -1 -> 1,      n -> n - 2   (n >= 2: the reference divides by zero
//                                       for n == 1, which the host refuses);
// `constant` reads `fill` when the index is out of range (genBnd2D,
// Lowering.hs:2842-2870).  Interior points read their neighbours directly.
enum { BND_CLAMP = 0, BND_WRAP = 1, BND_MIRROR = 2, BND_CONST = 3 };

template <int KIND, int BND>
__global__ void __launch_bounds__(256) stencil_bnd_kernel(const double* __restrict__ in, double* __restrict__ out,
                                                          int64_t h, int64_t w, double fill) {
    const int64_t j = (int64_t)blockIdx.x * 32 + (threadIdx.x & 31);
    const int64_t i = (int64_t)blockIdx.y * 8 + (threadIdx.x >> 5);
    if (i >= h || j >= w) return;
    const double e = in[i * w + j];
    double a, b, c, d;
    if (i > 0 && i + 1 < h && j > 0 && j + 1 < w) {
        a = in[(i - 1) * w + j];
        b = in[(i + 1) * w + j];
        c = in[i * w + j - 1];
        d = in[i * w + j + 1];
    } else if (BND == BND_CONST) {
        a = i > 0 ? in[(i - 1) * w + j] : fill;
        b = i + 1 < h ? in[(i + 1) * w + j] : fill;
        c = j > 0 ? in[i * w + j - 1] : fill;
        d = j + 1 < w ? in[i * w + j + 1] : fill;
    } else {
        const int64_t im = i > 0 ? i - 1 : (BND == BND_WRAP ? h - 1 : 1);
        const int64_t ip = i + 1 < h ? i + 1 : (BND == BND_WRAP ? 0 : h - 2);
        const int64_t jm = j > 0 ? j - 1 : (BND == BND_WRAP ? w - 1 : 1);
        const int64_t jp = j + 1 < w ? j + 1 : (BND == BND_WRAP ? 0 : w - 2);
        a = in[im * w + j];
        b = in[ip * w + j];
        c = in[i * w + jm];
        d = in[i * w + jp];
    }
    out[i * w + j] = stencil_body<KIND, 2>(a, b, c, d, e);
}

template <int KIND>
static int launch_bnd_kind(int bnd, double fill, const double* in, double* out, int64_t h, int64_t w,
                           cudaStream_t s) {
    const dim3 grid((unsigned)((w + 31) / 32), (unsigned)((h + 7) / 8));
    switch (bnd) {
        case BND_WRAP: stencil_bnd_kernel<KIND, BND_WRAP><<<grid, 256, 0, s>>>(in, out, h, w, fill); break;
        case BND_MIRROR: stencil_bnd_kernel<KIND, BND_MIRROR><<<grid, 256, 0, s>>>(in, out, h, w, fill); break;
        default: stencil_bnd_kernel<KIND, BND_CONST><<<grid, 256, 0, s>>>(in, out, h, w, fill); break;
    }
    return launch_check("stencil2d_bnd");
}

static int launch_bnd(int kind, int bnd, double fill, const double* in, double* out, int64_t h, int64_t w,
                      cudaStream_t s) {
    switch (kind) {
        case ST_LAPLACIAN: return launch_bnd_kind<ST_LAPLACIAN>(bnd, fill, in, out, h, w, s);
        case ST_JACOBI: return launch_bnd_kind<ST_JACOBI>(bnd, fill, in, out, h, w, s);
        case ST_HEAT: return launch_bnd_kind<ST_HEAT>(bnd, fill, in, out, h, w, s);
        default: return launch_bnd_kind<ST_HEAT_EXAMPLE>(bnd, fill, in, out, h, w, s);
    }
}

// Cached executable graphs of whole `iterate` runs (`fill`: the constant of a
// `constant` boundary, baked into the captured launches).
struct GraphKey {
    int kind;
    int64_t h, w, iters;
    const void *b0, *b1;
    cudaStream_t stream;
    double fill;
    bool operator<(const GraphKey& o) const {
        return std::tie(kind, h, w, iters, b0, b1, stream, fill) <
               std::tie(o.kind, o.h, o.w, o.iters, o.b0, o.b1, o.stream, o.fill);
    }
};
static std::mutex g_graph_mu;
static std::map<GraphKey, cudaGraphExec_t> g_graphs;

}  // namespace hyd

using namespace hyd;

extern "C" int hyd_cuda_stencil2d_f64_variant(int kind, const double* in, double* out, int64_t h, int64_t w,
                                              int variant, void* stream) {
    HYD_CHECK_ARG(kind >= 0 && kind <= 3, "stencil2d: unknown kind %d", kind);
    HYD_CHECK_ARG(h >= 0 && w >= 0, "stencil2d: negative shape");
    HYD_CHECK_ARG(h * w == 0 || (in != nullptr && out != nullptr), "stencil2d: null buffer");
    HYD_CHECK_ARG(in != out || h * w == 0, "stencil2d: input and output must differ");
    HYD_CHECK_ARG(variant >= -1 && variant < kNumVariants, "stencil2d: unknown variant %d", variant);
    if (h == 0 || w == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    const int v = choose_variant(kind, in, nullptr, h, w, variant);
    CUtensorMap map;
    HYD_TRY(maps_for(v, in, h, w, &map));
    return launch_step(kind, &map, in, out, h, w, v, d, as_stream(stream));
}

extern "C" int hyd_cuda_stencil2d_f64(int kind, const double* in, double* out, int64_t h, int64_t w,
                                      void* stream) {
    return hyd_cuda_stencil2d_f64_variant(kind, in, out, h, w, -1, stream);
}

extern "C" int hyd_cuda_iterate_stencil2d_f64_variant(int kind, double* buf0, double* buf1, int64_t h, int64_t w,
                                                      int64_t iters, int variant, int* final_buf, void* stream) {
    HYD_CHECK_ARG(kind >= 0 && kind <= 3, "iterate_stencil2d: unknown kind %d", kind);
    HYD_CHECK_ARG(h >= 0 && w >= 0 && iters >= 0, "iterate_stencil2d: negative shape or count");
    HYD_CHECK_ARG(final_buf != nullptr, "iterate_stencil2d: null final_buf");
    HYD_CHECK_ARG(h * w == 0 || (buf0 != nullptr && buf1 != nullptr && buf0 != buf1),
                  "iterate_stencil2d: need two distinct buffers");
    HYD_CHECK_ARG(variant >= -1 && variant < kNumVariants, "iterate_stencil2d: unknown variant %d", variant);
    *final_buf = (int)(iters & 1);
    if (h == 0 || w == 0 || iters == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    cudaStream_t st = as_stream(stream);
    const int v = choose_variant(kind, buf0, buf1, h, w, variant);
    CUtensorMap maps[2];
    HYD_TRY(maps_for(v, buf0, h, w, &maps[0]));
    HYD_TRY(maps_for(v, buf1, h, w, &maps[1]));
    double* bufs[2] = {buf0, buf1};
    // Graph capture needs a non-default stream; on the legacy stream run eagerly.
    if (st == nullptr || iters < 4) {
        for (int64_t t = 0; t < iters; ++t)
            HYD_TRY(launch_step(kind, &maps[t & 1], bufs[t & 1], bufs[(t + 1) & 1], h, w, v, d, st));
        return HYD_CUDA_OK;
    }
    GraphKey key{kind * 256 + v, h, w, iters, buf0, buf1, st, 0.0};
    cudaGraphExec_t exec = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_graph_mu);
        auto it = g_graphs.find(key);
        if (it != g_graphs.end()) exec = it->second;
    }
    if (!exec) {
        // warm the per-kernel configuration outside capture
        HYD_TRY(launch_step(kind, &maps[0], bufs[0], bufs[1], h, w, v, d, st));
        HYD_CUDA_TRY(cudaStreamSynchronize(st));
        cudaGraph_t graph = nullptr;
        HYD_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int status = HYD_CUDA_OK;
        for (int64_t t = 0; t < iters && status == HYD_CUDA_OK; ++t)
            status = launch_step(kind, &maps[t & 1], bufs[t & 1], bufs[(t + 1) & 1], h, w, v, d, st);
        cudaError_t ce = cudaStreamEndCapture(st, &graph);
        if (status != HYD_CUDA_OK) {
            if (graph) cudaGraphDestroy(graph);
            return status;
        }
        HYD_CUDA_TRY(ce);
        cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        HYD_CUDA_TRY(ie);
        std::lock_guard<std::mutex> lock(g_graph_mu);
        if (g_graphs.size() >= 64) {  // bounded cache: drop everything when full
            for (auto& kv : g_graphs) cudaGraphExecDestroy(kv.second);
            g_graphs.clear();
        }
        g_graphs[key] = exec;
    }
    HYD_CUDA_TRY(cudaGraphLaunch(exec, st));
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_iterate_stencil2d_f64(int kind, double* buf0, double* buf1, int64_t h, int64_t w,
                                              int64_t iters, int* final_buf, void* stream) {
    return hyd_cuda_iterate_stencil2d_f64_variant(kind, buf0, buf1, h, w, iters, -1, final_buf, stream);
}

static int check_bnd(int kind, int boundary, int64_t h, int64_t w, const char* what) {
    HYD_CHECK_ARG(kind >= 0 && kind <= 3, "%s: unknown kind %d", what, kind);
    HYD_CHECK_ARG(boundary >= HYD_BOUNDARY_CLAMP && boundary <= HYD_BOUNDARY_CONSTANT, "%s: unknown boundary %d",
                  what, boundary);
    HYD_CHECK_ARG(h >= 0 && w >= 0, "%s: negative shape", what);
    HYD_CHECK_ARG(boundary != HYD_BOUNDARY_MIRROR || h * w == 0 || (h >= 2 && w >= 2),
                  "%s: a mirror boundary needs every extent >= 2 (%lld x %lld; the reference divides by zero)",
                  what, (long long)h, (long long)w);
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_stencil2d_bnd_f64(int kind, int boundary, double fill, const double* in, double* out,
                                          int64_t h, int64_t w, void* stream) {
    HYD_TRY(check_bnd(kind, boundary, h, w, "stencil2d_bnd"));
    if (boundary == HYD_BOUNDARY_CLAMP) return hyd_cuda_stencil2d_f64(kind, in, out, h, w, stream);
    HYD_CHECK_ARG(h * w == 0 || (in != nullptr && out != nullptr), "stencil2d_bnd: null buffer");
    HYD_CHECK_ARG(in != out || h * w == 0, "stencil2d_bnd: input and output must differ");
    if (h == 0 || w == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    return launch_bnd(kind, boundary, fill, in, out, h, w, as_stream(stream));
}

extern "C" int hyd_cuda_iterate_stencil2d_bnd_f64(int kind, int boundary, double fill, double* buf0, double* buf1,
                                                  int64_t h, int64_t w, int64_t iters, int* final_buf,
                                                  void* stream) {
    HYD_TRY(check_bnd(kind, boundary, h, w, "iterate_stencil2d_bnd"));
    if (boundary == HYD_BOUNDARY_CLAMP)
        return hyd_cuda_iterate_stencil2d_f64(kind, buf0, buf1, h, w, iters, final_buf, stream);
    HYD_CHECK_ARG(iters >= 0 && final_buf != nullptr, "iterate_stencil2d_bnd: bad count or null final_buf");
    HYD_CHECK_ARG(h * w == 0 || (buf0 != nullptr && buf1 != nullptr && buf0 != buf1),
                  "iterate_stencil2d_bnd: need two distinct buffers");
    *final_buf = (int)(iters & 1);
    if (h == 0 || w == 0 || iters == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    cudaStream_t st = as_stream(stream);
    double* bufs[2] = {buf0, buf1};
    if (st == nullptr || iters < 4) {
        for (int64_t t = 0; t < iters; ++t)
            HYD_TRY(launch_bnd(kind, boundary, fill, bufs[t & 1], bufs[(t + 1) & 1], h, w, st));
        return HYD_CUDA_OK;
    }
    // keys of this form sit above the clamp path's kind * 256 + variant (< 256)
    GraphKey key{1024 + kind * 4 + boundary, h, w, iters, buf0, buf1, st, fill};
    cudaGraphExec_t exec = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_graph_mu);
        auto it = g_graphs.find(key);
        if (it != g_graphs.end()) exec = it->second;
    }
    if (!exec) {
        cudaGraph_t graph = nullptr;
        HYD_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int status = HYD_CUDA_OK;
        for (int64_t t = 0; t < iters && status == HYD_CUDA_OK; ++t)
            status = launch_bnd(kind, boundary, fill, bufs[t & 1], bufs[(t + 1) & 1], h, w, st);
        cudaError_t ce = cudaStreamEndCapture(st, &graph);
        if (status != HYD_CUDA_OK) {
            if (graph) cudaGraphDestroy(graph);
            return status;
        }
        HYD_CUDA_TRY(ce);
        cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        HYD_CUDA_TRY(ie);
        std::lock_guard<std::mutex> lock(g_graph_mu);
        if (g_graphs.size() >= 64) {
            for (auto& kv : g_graphs) cudaGraphExecDestroy(kv.second);
            g_graphs.clear();
        }
        g_graphs[key] = exec;
    }
    HYD_CUDA_TRY(cudaGraphLaunch(exec, st));
    return HYD_CUDA_OK;
}

namespace hyd {
void release_more_graphs();  // stencil_more.cu
}

extern "C" void hyd_cuda_stencil_release_graphs(void) {
    {
        std::lock_guard<std::mutex> lock(g_graph_mu);
        for (auto& kv : g_graphs) cudaGraphExecDestroy(kv.second);
        g_graphs.clear();
    }
    release_more_graphs();
}

// ---------------------------------------------------------------- self-test
namespace hyd {
__global__ void dadd_selftest_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                     double* __restrict__ emu, double* __restrict__ hw, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        emu[i] = dadd_pos(x[i], y[i]);
        hw[i] = __dadd_rn(x[i], y[i]);
    }
}
}  // namespace hyd

__global__ void div_selftest_kernel(const double* __restrict__ x, int divisor, double* __restrict__ fast,
                                    double* __restrict__ hw, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        fast[i] = divisor == 3 ? ddiv_small_rn<3>(x[i]) : ddiv_small_rn<5>(x[i]);
        hw[i] = __ddiv_rn(x[i], (double)divisor);
    }
}

extern "C" int hyd_cuda_selftest_div(const double* x, int divisor, double* fast, double* hw, int64_t n,
                                     void* stream) {
    HYD_CHECK_ARG(n >= 0 && (n == 0 || (x && fast && hw)), "selftest_div: bad arguments");
    HYD_CHECK_ARG(divisor == 3 || divisor == 5, "selftest_div: divisor must be 3 or 5 (got %d)", divisor);
    if (n == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    const int64_t want = (n + 255) / 256;
    const unsigned grid = (unsigned)(want < (int64_t)d->sm_count * 8 ? want : (int64_t)d->sm_count * 8);
    div_selftest_kernel<<<grid, 256, 0, as_stream(stream)>>>(x, divisor, fast, hw, n);
    return launch_check("selftest_div");
}

extern "C" int hyd_cuda_selftest_dadd(const double* x, const double* y, double* emu, double* hw, int64_t n,
                                      void* stream) {
    HYD_CHECK_ARG(n >= 0 && (n == 0 || (x && y && emu && hw)), "selftest_dadd: bad arguments");
    if (n == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    const int64_t want = (n + 255) / 256;
    const unsigned grid = (unsigned)(want < (int64_t)d->sm_count * 8 ? want : (int64_t)d->sm_count * 8);
    dadd_selftest_kernel<<<grid, 256, 0, as_stream(stream)>>>(x, y, emu, hw, n);
    return launch_check("selftest_dadd");
}
