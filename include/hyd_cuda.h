/* include/hyd_cuda.h -- C ABI of the GB300 (sm_103a) CUDA runtime for the
 * Hydrangea fused-loop hot path.
 *
 * Two layers:
 *   1. Device primitives on raw device pointers and a CUDA stream (cudaStream_t
 *      passed as void*; NULL = the legacy default stream).  These are the calls
 *      that host code generated for `--backend cuda` makes for each fused loop
 *      nest, one per loop template of the reference C backend.
 *   2. The embedding boundary on `hyd_array_t*` (the reference runtime's array
 *      ABI, unchanged): lifecycle `hyd_cuda_init` / `hyd_cuda_cleanup` in the
 *      style of the Metal backend's exported lifecycle, and `hyd_export_*`
 *      symbols with the signatures the reference's export wrapper gives the
 *      benchmark programs.
 *
 * Every function returns a hyd_cuda_status_t (0 = success) unless stated
 * otherwise; hyd_cuda_last_error() describes the most recent failure on the
 * calling thread.  Argument checks happen before any CUDA call, so a bad call
 * fails the same way with or without a GPU.
 *
 * Reference citations are file:line in hydrangea-compiler.
 */
#ifndef HYD_CUDA_H
#define HYD_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- array ABI -------------------------------------------------------------
 * Layout-identical to hyd_tuple_t / hyd_array_storage_t / hyd_array_t of
 * runtime/hydrangea_runtime.h:220-235.  When that header was included first its
 * definitions are used; otherwise these stand in (the refcount is a plain
 * int64_t here: same size and alignment as the header's _Atomic int64_t). */
#ifndef HYDRANGEA_RUNTIME_H
#define HYD_MAX_DIMS 8
typedef struct {
    int64_t elems[HYD_MAX_DIMS];
    int ndims;
} hyd_tuple_t;
typedef struct {
    unsigned char* data;
    int64_t refcount;
} hyd_array_storage_t;
typedef struct {
    hyd_array_storage_t* storage;
    unsigned char* data;
    size_t elem_size;
    hyd_tuple_t shape;
} hyd_array_t;
#endif

typedef enum {
    HYD_CUDA_OK = 0,
    HYD_CUDA_ERR_INVALID = 1,     /* bad argument (null pointer, negative size, ...) */
    HYD_CUDA_ERR_NOMEM = 2,       /* device or host allocation failed */
    HYD_CUDA_ERR_CUDA = 3,        /* a CUDA runtime/driver call failed */
    HYD_CUDA_ERR_NO_DEVICE = 4,   /* no usable GPU */
    HYD_CUDA_ERR_BOUNDS = 5,      /* a route/index left its destination (device-detected) */
    HYD_CUDA_ERR_TIMEOUT = 6,     /* a bounded device wait gave up */
    HYD_CUDA_ERR_BUDGET = 7,      /* serving: request exceeds the HBM budget */
    HYD_CUDA_ERR_CANCELLED = 8,   /* serving: request cancelled or server stopped */
    HYD_CUDA_ERR_UNSUPPORTED = 9  /* shape/size outside what this build supports */
} hyd_cuda_status_t;

/* ---- lifecycle (the Metal backend's exported hyd_metal_init/_cleanup pair,
 *      CodegenMSL.hs:1219-1222, re-targeted at CUDA) ------------------------ */
int hyd_cuda_init(void);                 /* 0 on success; idempotent */
void hyd_cuda_cleanup(void);             /* frees runtime-owned device memory */
const char* hyd_cuda_last_error(void);   /* thread-local message of the last failure */
const char* hyd_cuda_status_string(int status);
int hyd_cuda_version(void);              /* ABI version, major*100 + minor */
int hyd_cuda_device_sm_count(void);      /* SMs of the current device, or -status */
/* Synchronize `stream`, then report (and clear) device-detected errors such as
 * out-of-range scatter routes raised by kernels launched since the last check. */
int hyd_cuda_check(void* stream);

/* ---- seeded synthetic inputs (same counter-based SplitMix64 stream as the
 *      CPU oracle; element i depends only on (seed, i)) ---------------------- */
int hyd_cuda_fill_uniform_f64(double* out, int64_t n, uint64_t seed, double lo, double hi,
                              void* stream);
int hyd_cuda_fill_uniform_i64(int64_t* out, int64_t n, uint64_t seed, int64_t bound,
                              void* stream);

/* ---- reduce (+) 0.0 (zipwith (*) xs ys) -----------------------------------
 * Replaces the parallel reduction template CodegenC.hs:1328-1353 (emitted
 * `omp parallel for simd reduction(+:acc)`, README.md:25-33) for the fused
 * reduce_generate of Lowering.hs:771-804.  Deterministic: a fixed grid, per
 * thread fixed-order accumulation, warp-shuffle trees and a fixed-order final
 * combine, so the same inputs give the same bits on every run.  *out is a
 * device pointer to one double. */
int hyd_cuda_dot_f64(const double* xs, const double* ys, int64_t n, double* out, void* stream);
/* reduce (+) 0.0 xs, same scheme. */
int hyd_cuda_sum_f64(const double* xs, int64_t n, double* out, void* stream);
/* hyd_cuda_dot_f64 for callers that must not allocate device memory (no
 * counterpart in the reference; it exists for hosts where cudaMalloc may stall
 * other streams or fail under a fixed memory budget).  Same kernel and same
 * result bits, but its scratch lives in a static device array inside this
 * library (about 16 KiB, held on every GPU that loads the library until exit)
 * instead of a runtime-allocated workspace.  Calls no cudaMalloc/cudaFree and
 * no allocating library routine.  Limit: at most 2048 CTAs of partials (two per
 * SM), otherwise HYD_CUDA_ERR_UNSUPPORTED.  The first call on each device looks
 * up the array's device address; make that first call before any stream
 * capture.  All calls share the one array: calls that overlap on the GPU (for
 * example on two streams at once) race and give wrong results. */
int hyd_cuda_dot_f64_noalloc(const double* xs, const double* ys, int64_t n, double* out, void* stream);

/* ---- scatter (+) ------------------------------------------------------------
 * Replaces the privatized scatter template CodegenC.hs:1119-1288 and the
 * atomic template CodegenC.hs:1084-1118 (strategy choice Parallelize.hs:
 * 466-503).  Fused weighted histogram of examples/weighted_histogram.hyd:
 *   hist[x % bins] += x * x   for x in data   (int64, wrapping)
 * `hist` (device, bins int64) is accumulated into, like the reference's
 * merge into the existing destination; zero it first for `fill [bins] 0`.
 * A route outside [0, bins) is skipped and reported by hyd_cuda_check. */
typedef enum {
    HYD_SCATTER_AUTO = 0,          /* autotuned choice per (bins class) */
    HYD_SCATTER_SMEM_WARP = 1,     /* per-warp shared-memory bins */
    HYD_SCATTER_SMEM_BLOCK = 2,    /* one shared-memory copy per block */
    HYD_SCATTER_CLUSTER = 3,       /* bins spread over a thread-block cluster's DSMEM */
    HYD_SCATTER_GLOBAL = 4,        /* global atomics (bins beyond on-chip memory) */
    HYD_SCATTER_PARTITION = 5      /* staging pass grouping elements by bin range, then one
                                      shared-memory pass per range (single-word sources) */
} hyd_scatter_strategy_t;
int hyd_cuda_weighted_histogram_i64(const int64_t* data, int64_t n, int64_t bins,
                                    int64_t* hist, int strategy, void* stream);
/* The strategy a weighted_histogram call of this shape runs (AUTO resolved,
 * tuned choices included) and how many kernels it launches.  No counterpart
 * in the reference; for reporting and tests. */
int hyd_cuda_weighted_histogram_plan(int64_t n, int64_t bins, int strategy, int* chosen, int* launches);
/* Unfused scatter (+) over materialised routes and values (Lowering.hs:
 * 1408-1430): dst[idx[i]] += vals[i].  int64 variant is order-independent
 * (bit-exact); the float variant accumulates with fp64 atomics and is
 * therefore run-to-run order-dependent within fp64 rounding. */
int hyd_cuda_scatter_add_i64(const int64_t* idx, const int64_t* vals, int64_t n,
                             int64_t* dst, int64_t dst_n, int strategy, void* stream);
int hyd_cuda_scatter_add_f64(const int64_t* idx, const double* vals, int64_t n,
                             double* dst, int64_t dst_n, void* stream);
/* A scatter (+) phase with a guard (Lowering.hs:1768-1790): element i takes
 * part only when guard[i] != 0 (its index is not read otherwise).  Every
 * strategy of the weighted histogram serves it; bit-exact. */
int hyd_cuda_scatter_add_guarded_i64(const int64_t* idx, const int64_t* vals, const int64_t* guard, int64_t n,
                                     int64_t* dst, int64_t dst_n, int strategy, void* stream);

/* `reduce` over the trailing axis of an array [rows, cols] (EReduce,
 * Lowering.hs:723-760): out[j] = init `op` x[j,0] `op` ... `op` x[j,cols-1],
 * op one of the reference's reduction operators (CFGCore.hs:236).  int64
 * wraps and is exact; f64 rows of up to 32 elements fold in the reference's
 * order (bit-identical), longer ones by a fixed tree (deterministic, within
 * rounding of the serial fold). */
enum { HYD_REDOP_ADD = 0, HYD_REDOP_MUL = 1 };
int hyd_cuda_reduce_rows_i64(const int64_t* in, int64_t rows, int64_t cols, int op, int64_t init, int64_t* out,
                             void* stream);
int hyd_cuda_reduce_rows_f64(const double* in, int64_t rows, int64_t cols, int op, double init, double* out,
                             void* stream);

/* ---- 2-D clamp stencils and iterate ---------------------------------------
 * Replaces the split-region clamp stencil loops (Lowering.hs:1932-2035,
 * :2562-2661; each region an `omp parallel for`) and the ping-pong iterate
 * (Lowering.hs:840-858, CFGOpt.hs:795-810).  5-point footprint, clamp-to-edge,
 * row-major float64 [h][w].  Bodies, evaluated left to right as the program
 * text (a = acc (-1) 0, b = acc 1 0, c = acc 0 (-1), d = acc 0 1, e = acc 0 0):
 *   HYD_STENCIL_LAPLACIAN     a + b + c + d + (e * -4.0)    bench/stencil/stencil_2d.hyd
 *   HYD_STENCIL_JACOBI        (a + b + c + d) / 4.0          bench/stencil/jacobi_2d.hyd
 *   HYD_STENCIL_HEAT          e + 0.1 * (a+b+c+d - 4.0*e)    heat step of the 8192^2 workload
 *   HYD_STENCIL_HEAT_EXAMPLE  (a + b + c + d + e) / 5.0      examples/heat_2d.hyd
 * Results are bit-identical to the C backend. */
typedef enum {
    HYD_STENCIL_LAPLACIAN = 0,
    HYD_STENCIL_JACOBI = 1,
    HYD_STENCIL_HEAT = 2,
    HYD_STENCIL_HEAT_EXAMPLE = 3
} hyd_stencil_kind_t;
int hyd_cuda_stencil2d_f64(int kind, const double* in, double* out, int64_t h, int64_t w, void* stream);
/* iterate iters (stencil kind) over buf0 with ping-pong into buf1; *final_buf
 * is set to the buffer (0 or 1) holding the result.  On a non-default stream
 * the whole run is a captured CUDA graph, cached per (kind, shape, buffers,
 * iters, stream) and replayed on later calls. */
int hyd_cuda_iterate_stencil2d_f64(int kind, double* buf0, double* buf1, int64_t h, int64_t w,
                                   int64_t iters, int* final_buf, void* stream);
/* The same kinds under the other boundary conditions of `stencil`
 * (Syntax.hs:416-426): the neighbour index per dimension as the reference's
 * lowering computes it (Lowering.hs:2762-2870) -- wrap: periodic; mirror:
 * reflected without repeating the edge (every extent must be >= 2: the
 * reference divides by zero otherwise, HYD_CUDA_ERR_INVALID here); constant:
 * `fill` outside the array.  HYD_BOUNDARY_CLAMP takes the functions above. */
enum { HYD_BOUNDARY_CLAMP = 0, HYD_BOUNDARY_WRAP = 1, HYD_BOUNDARY_MIRROR = 2, HYD_BOUNDARY_CONSTANT = 3 };
int hyd_cuda_stencil2d_bnd_f64(int kind, int boundary, double fill, const double* in, double* out, int64_t h,
                               int64_t w, void* stream);
int hyd_cuda_iterate_stencil2d_bnd_f64(int kind, int boundary, double fill, double* buf0, double* buf1, int64_t h,
                                       int64_t w, int64_t iters, int* final_buf, void* stream);
/* Self-test of the integer-pipe binary64 addition the stencil variants of
 * levels 1-2 use: emu[i] = that addition of x[i] and y[i], hw[i] = the FP64
 * unit's x[i] + y[i] (round to nearest even).  No counterpart in the
 * reference; for tests. */
int hyd_cuda_selftest_dadd(const double* x, const double* y, double* emu, double* hw, int64_t n, void* stream);
/* Self-test of the multiply-and-two-FMA division by 3 or 5 that jacobi_1d and
 * the heat example's 5-point mean use: fast[i] = that quotient x[i] / divisor,
 * hw[i] = the IEEE division (round to nearest even).  No counterpart in the
 * reference; for tests. */
int hyd_cuda_selftest_div(const double* x, int divisor, double* fast, double* hw, int64_t n, void* stream);
/* Issue-rate probe of the FP64 unit: a kernel of sm_count x 4 blocks of 256
 * threads, each running `iters` rounds of 8 independent fma chains, so that
 * the FP64 pipe, not latency, bounds it.  *fma_count (HOST, may be NULL)
 * receives the number of fma operations launched; the caller times the launch
 * with CUDA events on `stream` and divides.  sink: two device doubles.  No
 * counterpart in the reference; it supplies the measured denominator of the
 * FP64-bound kernels' roofline. */
int hyd_cuda_probe_fp64_rate(int64_t iters, double* sink, int64_t* fma_count, void* stream);
/* Timeout self-test: runs one of the runtime's bounded device waits on a
 * condition that nothing ever satisfies, with at most poll_limit (1..2^20)
 * polls, so that it gives up.  which = 0: the mbarrier wait of the TMA kernels;
 * which = 1: the tile-status wait of the decoupled look-back scans.  The wait
 * sets the device error word exactly as a real timeout does: the next
 * hyd_cuda_check(stream) returns HYD_CUDA_ERR_TIMEOUT, and the device stays
 * usable.  No counterpart in the reference; for tests. */
int hyd_cuda_selftest_timeout(int which, uint32_t poll_limit, void* stream);
/* ---- fused map / zipwith / generate chains -------------------------------------
 * The element loop of a fused chain (bench/map_chain/map_chain.hyd; the C
 * backend's loop body, CodegenC.hs:1328-1353 for the reduced form) with its
 * body given as generated C statements over x0..x{ninputs-1} (element i of
 * inputs[k], double), i (int64 index) and assigning the double `v`, e.g.
 *   "double s = (double)i / 4096.0; double a = s * s; v = (a - 0.5) * 2.0 + 1.0;"
 * inputs: HOST array of ninputs (<= 8) device pointers.  out (n doubles, may be
 * NULL) receives the elements, each bit-identical to the C backend (IEEE
 * round-to-nearest, no contraction); sum (one device double, may be NULL)
 * receives their (+) reduction in a fixed order (run-to-run identical).
 * Compiled once per (device, body, ninputs) at run time with NVRTC
 * (HYD_CUDA_ERR_UNSUPPORTED if the NVRTC library is absent; a body that does
 * not compile is HYD_CUDA_ERR_INVALID with the compiler's message). */
int hyd_cuda_map_f64(const char* body, const double* const* inputs, int ninputs, int64_t n, double* out,
                     double* sum, void* stream);
/* The same for int64 elements (x0..x7, v and the (+) reduction int64): the
 * generated body keeps C's int64 semantics (truncating / and %); the sum
 * wraps mod 2^64 and is bit-exact. */
int hyd_cuda_map_i64(const char* body, const int64_t* const* inputs, int ninputs, int64_t n, int64_t* out,
                     int64_t* sum, void* stream);

/* ---- the other iterate loops ---------------------------------------------------
 * jacobi_1d (examples/jacobi_1d.hyd:4): out[i] = (in[i-1] + in[i] + in[i+1]) / 3.0
 * with clamped neighbours, float64, bit-identical to the C backend. */
int hyd_cuda_jacobi1d_f64(const double* in, double* out, int64_t n, void* stream);
int hyd_cuda_iterate_jacobi1d_f64(double* buf0, double* buf1, int64_t n, int64_t iters, int* final_buf,
                                  void* stream);
/* Gray-Scott reaction-diffusion (demo/gray_scott/gray_scott.hyd:47-73): one step
 * of U and V on an h x w periodic grid, each expression in the program's order
 * (bit-identical to the C backend).  params NULL = the demo's constants
 * (du 0.21, dv 0.105, feed 0.0545, kill 0.0620, dt 1.0).  The iterate form
 * ping-pongs (u0, v0) <-> (u1, v1); *final_buf = 1 when the result is in
 * (u1, v1).  Like the stencil iterate, a non-default stream runs a cached
 * captured graph. */
typedef struct {
    double du, dv, feed, kill, dt;
} hyd_gray_scott_t;
int hyd_cuda_gray_scott_step_f64(const double* u, const double* v, double* u_out, double* v_out, int64_t h,
                                 int64_t w, const hyd_gray_scott_t* params, void* stream);
int hyd_cuda_iterate_gray_scott_f64(double* u0, double* v0, double* u1, double* v1, int64_t h, int64_t w,
                                    const hyd_gray_scott_t* params, int64_t steps, int* final_buf, void* stream);
/* Releases the cached iterate graphs (also done by hyd_cuda_cleanup). */
void hyd_cuda_stencil_release_graphs(void);
/* Same, with an explicit kernel variant instead of the autotuned one
 * (-1 = autotuned/default).  variant = shape + 7 * level.  Shapes 0..5 are
 * TMA tile shapes (0 = 32x32, the reference's fixed polyhedral tile,
 * Polyhedral.hs:196-204; 1 = 16x128, 2 = 16x64, 3 = 32x64, 4 = 8x128,
 * 5 = 32x128), 6 = the plain non-TMA kernel.  Levels 0, 1, 2 run 0, 2, 3 of
 * the three additions of the 4-neighbour sum on the integer pipe (exact
 * round-to-nearest-even; FP64 is the scarce pipe on GB300).  All 21 variants
 * give identical bits. */
int hyd_cuda_stencil2d_f64_variant(int kind, const double* in, double* out, int64_t h, int64_t w,
                                   int variant, void* stream);
int hyd_cuda_iterate_stencil2d_f64_variant(int kind, double* buf0, double* buf1, int64_t h, int64_t w,
                                           int64_t iters, int variant, int* final_buf, void* stream);

/* ---- autotuner ---------------------------------------------------------------
 * Chooses, per (kernel, shape class), the fastest of candidates that all give
 * identical results, measuring on the current device; choices persist in a
 * tab-separated cache (HYD_CUDA_TUNE_CACHE, default
 * $HOME/.cache/hydrangea_cuda_tune.tsv) and are consulted by AUTO launches.
 * Shape classes: stencil2d "k<kind>_h<log2 h>_w<log2 w>", weighted_histogram
 * "b<log2 bins>" (ceil log2). */
const char* hyd_cuda_tune_cache_path(void);
int hyd_cuda_tune_set_cache_path(const char* path);     /* reloads the table from `path` */
int hyd_cuda_tune_record(const char* device, const char* kernel, const char* klass, int choice, double us);
int hyd_cuda_tune_query(const char* device, const char* kernel, const char* klass);  /* -1 if absent */
/* Time every stencil variant (times_us[21], may be NULL) / histogram strategy
 * (times_us[6], index = strategy, -1 when it cannot run) on scratch inputs and
 * record the fastest in *best. */
int hyd_cuda_autotune_stencil2d(int kind, int64_t h, int64_t w, int reps, int* best, double* times_us);
int hyd_cuda_autotune_histogram(int64_t n, int64_t bins, int reps, int* best, double* times_us);

/* ---- scan family and segmented reduce ----------------------------------------
 * scan / scan_inclusive / scanr / scanr_inclusive with (+) and initial value
 * `init` (Lowering.hs:3563-3612; the reference runs them as a serial fold):
 * reverse != 0 walks index n-1-k; inclusive != 0 writes the accumulator after
 * adding element k, otherwise before.  int64: single-pass decoupled look-back,
 * bit-exact.  float64: single pass, deterministic (a fixed warp scan within
 * blocks of 32 tiles, a left fold of the block totals): run-to-run identical
 * and within 1e-12 of the prefix sums of |x| of the serial fold. */
int hyd_cuda_scan_i64(const int64_t* in, int64_t* out, int64_t n, int64_t init, int reverse,
                      int inclusive, void* stream);
int hyd_cuda_scan_f64(const double* in, double* out, int64_t n, double init, int reverse,
                      int inclusive, void* stream);
/* segmented_reduce (+) init offsets vals (Lowering.hs:874-944): out[s] = init +
 * sum of vals[offsets[s] .. offsets[s+1]).  n_offsets = segments + 1.  A
 * segment outside [0, n_vals] or with decreasing offsets yields init and is
 * reported by hyd_cuda_check.  int64 bit-exact; float64 deterministic, within
 * 1e-12 of the sum of |vals| of the segment. */
int hyd_cuda_segmented_reduce_i64(const int64_t* offsets, int64_t n_offsets, const int64_t* vals,
                                  int64_t n_vals, int64_t init, int64_t* out, void* stream);
int hyd_cuda_segmented_reduce_f64(const int64_t* offsets, int64_t n_offsets, const double* vals,
                                  int64_t n_vals, double init, double* out, void* stream);

/* ---- sort_indices and gather ---------------------------------------------------
 * sort_indices keys (runtime/hydrangea_runtime.h:386-456): the permutation
 * that stably sorts `keys` by the runtime's LSD radix digits ((key >> 8p) &
 * 0xFF on the signed key, passes = bytes of max(0, max key), at least one), so
 * the permutation is identical to the reference runtime's.  perm is int64.
 * hyd_cuda_sort_indices_i64 finds the pass count on the device (one 8-byte
 * read-back); the _bits variant takes it from the caller (keys known to fit in
 * key_bits bits; same result when that bound holds). */
int hyd_cuda_sort_indices_i64(const int64_t* keys, int64_t n, int64_t* perm, void* stream);
int hyd_cuda_sort_indices_bits_i64(const int64_t* keys, int64_t n, int key_bits, int64_t* perm,
                                   void* stream);
/* gather perm src: out[i] = src[perm[i]]; an index outside [0, src_n) leaves
 * out[i] unwritten and is reported by hyd_cuda_check. */
int hyd_cuda_gather_i64(const int64_t* perm, int64_t n, const int64_t* src, int64_t src_n,
                        int64_t* out, void* stream);
int hyd_cuda_gather_f64(const int64_t* perm, int64_t n, const double* src, int64_t src_n,
                        double* out, void* stream);
int hyd_cuda_gather_i32(const int64_t* perm, int64_t n, const int32_t* src, int64_t src_n,
                        int32_t* out, void* stream);

/* ---- COO / CSR / SpMV ------------------------------------------------------------
 * coo_sum_duplicates (Lowering.hs:966-1080): merges adjacent entries with equal
 * (row, col) of a sorted COO, summing their int64 values.  Outputs have the
 * input's length; entries past the canonical count are zero, as in the
 * reference's calloc'd result.  *out_nnz (device int64) receives the count. */
int hyd_cuda_coo_sum_duplicates_i64(const int64_t* rows, const int64_t* cols, const int64_t* vals,
                                    int64_t nnz, int64_t* out_rows, int64_t* out_cols,
                                    int64_t* out_vals, int64_t* out_nnz, void* stream);
/* csr_from_sorted_coo (Lowering.hs:1081-1160): row_ptr[nrows+1] = exclusive
 * running sum of per-row counts (total last), col_idx/out_vals = the first
 * nnz cols/vals copied through.  A row outside [0, nrows) is reported by
 * hyd_cuda_check. */
int hyd_cuda_csr_from_sorted_coo_i64(int64_t nrows, int64_t nnz, const int64_t* rows,
                                     const int64_t* cols, const int64_t* vals, int64_t* row_ptr,
                                     int64_t* col_idx, int64_t* out_vals, void* stream);
/* SpMV y = A x over CSR (bench/spmv/spmv.hyd:30-40): lanes_per_row lanes (power
 * of two <= 32, 0 = default 8) share a row with fma partial sums and a fixed
 * xor tree: deterministic, within 1e-12 of sum |v*x| of the sequential C sum.
 * A column outside [0, ncols) is skipped and reported. */
int hyd_cuda_spmv_csr_f64(int64_t nrows, int64_t ncols, const int64_t* row_ptr, const int64_t* col_idx,
                          const double* vals, const double* x, double* y, int lanes_per_row, void* stream);
int hyd_cuda_spmv_csr_i32_f64(int64_t nrows, int64_t ncols, const int64_t* row_ptr,
                              const int32_t* col_idx, const double* vals, const double* x, double* y,
                              int lanes_per_row, void* stream);
/* Batched COO -> CSR -> SpMV over ninst instances in one persistent pass.
 * desc: HOST array of ninst x (nrows, ncols, nnz).  Device arrays are the
 * instances concatenated in order: rows/cols (int32, device narrowing of the
 * int64 ABI, valid for extents < 2^31), vals, csr_cols, csr_vals by entries;
 * x by ncols; y by nrows; row_ptr by nrows + 1 (each instance's row_ptr starts
 * at 0).  Per instance the CSR equals sorting the entries by (row, col) (the
 * packed-key pipeline of bench/coo_csr_build/coo_csr_build.hyd:37-62) and y is
 * its SpMV; equal (row, col) entries keep their COO order, as the runtime's
 * stable sort_indices leaves them.  Contract: at most 256 entries per row (the
 * workload's cap); a longer row or an out-of-range entry is reported by
 * hyd_cuda_check.  Synchronizes the stream before returning. */
int hyd_cuda_batched_coo_csr_spmv_f64(int64_t ninst, const int64_t* desc, const int32_t* rows,
                                      const int32_t* cols, const double* vals, const double* x,
                                      int64_t* row_ptr, int32_t* csr_cols, double* csr_vals, double* y,
                                      void* stream);
/* Seeded synthetic batch: ninst square instances, instance i from seed seed0+i
 * with n = floor(2^(min_log2 + (max_log2-min_log2) u)), rows of Zipf(1.5)
 * length on {1..max_row_len}, distinct columns, values and x uniform in
 * [-1, 1), entries stored in a shuffled order.  Always fills desc (HOST,
 * ninst x 3); when rows is NULL only the sizes are computed, otherwise
 * rows/cols/vals (capacity_entries) and x (sum of n) are filled. */
int hyd_cuda_synth_coo_batch(int64_t ninst, uint64_t seed0, int min_log2, int max_log2, int max_row_len,
                             int64_t* desc, int32_t* rows, int32_t* cols, double* vals, double* x,
                             int64_t capacity_entries, void* stream);

/* ---- serving --------------------------------------------------------------------
 * A resident request server inside the runtime (no reference counterpart; the
 * nearest are the memoised procedures of CodegenC.hs:690-707 and the Metal
 * export lifecycle with cached device buffers, CodegenMSL.hs:1120-1181).
 * Requests reference device-resident arrays.  Kinds and fields:
 *   HYD_REQ_DOT        n elements; in0 xs, in1 ys (f64); out0 one f64
 *   HYD_REQ_HIST       n elements, m bins (<= 8192); in0 data (i64); out0 hist
 *                      (m int64, overwritten): the fused weighted histogram
 *   HYD_REQ_LAPLACIAN  n rows, m cols; in0 grid, out0 grid (f64): one clamp
 *                      Laplacian step (HYD_STENCIL_LAPLACIAN)
 *   HYD_REQ_SPMV       n rows = cols, m entries; in0 rows, in1 cols (int32),
 *                      in2 vals, in3 x (f64); out0 y, out1 row_ptr (n+1 int64),
 *                      out2 csr cols (int32), out3 csr vals: COO -> CSR -> SpMV
 *                      as hyd_cuda_batched_coo_csr_spmv_f64 for one instance.
 * Admission: a request is admitted once the working sets in flight plus its own
 * fit hbm_budget_bytes (FIFO); a request larger than the budget completes with
 * HYD_CUDA_ERR_BUDGET.  Continuous batching: when a stream slot is free every
 * admitted waiting request (up to max_batch / max_batch_bytes) joins one batch,
 * dot/hist/Laplacian in a single persistent launch over (request, tile) work
 * items, SpMV requests in the batched pipeline; slots overlap on the device.
 * A request's result does not depend on what it was batched with.  Requests
 * that may be in flight together must not write the same output arrays (their
 * kernels would race, as any two overlapping launches would). */
typedef enum { HYD_REQ_DOT = 1, HYD_REQ_HIST = 2, HYD_REQ_LAPLACIAN = 3, HYD_REQ_SPMV = 4 } hyd_request_kind_t;
typedef struct {
    int kind;
    int64_t n;
    int64_t m;
    const void* in0;
    const void* in1;
    const void* in2;
    const void* in3;
    void* out0;
    void* out1;
    void* out2;
    void* out3;
} hyd_request_t;
typedef struct {
    int64_t hbm_budget_bytes;  /* 0: a quarter of the free device memory */
    int streams;               /* launch slots in flight (0: 4) */
    int max_batch;             /* requests per batch (0: 256) */
    int64_t max_batch_bytes;   /* working set per batch (0: budget / streams) */
} hyd_server_config_t;
typedef struct {
    int64_t submitted, completed, failed, rejected, cancelled;
    int64_t launches;             /* batches issued */
    int64_t peak_inflight_bytes;  /* never above hbm_budget_bytes */
    int64_t inflight_bytes, queued;
} hyd_server_stats_t;
typedef struct hyd_server hyd_server_t;
int hyd_cuda_server_create(const hyd_server_config_t* cfg, hyd_server_t** out);
/* Non-blocking; returns the request's immediate status (a validation, budget
 * or shutdown rejection) or HYD_CUDA_OK when queued.  *ticket is always set. */
int hyd_cuda_server_submit(hyd_server_t* srv, const hyd_request_t* req, int64_t* ticket);
/* Blocks until the ticket's request finished; status and latency
 * (arrival -> result ready, seconds). */
int hyd_cuda_server_wait(hyd_server_t* srv, int64_t ticket, int* status, double* latency_s);
int hyd_cuda_server_stats(hyd_server_t* srv, hyd_server_stats_t* out);
/* Message of the last batch that failed inside the server ("" if none). */
const char* hyd_cuda_server_error(hyd_server_t* srv);
/* Stops accepting work: queued requests complete with HYD_CUDA_ERR_CANCELLED,
 * batches in flight finish; tickets stay queryable until destroy. */
int hyd_cuda_server_shutdown(hyd_server_t* srv);
/* Shutdown (if not done) and release every resource of the server. */
int hyd_cuda_server_destroy(hyd_server_t* srv);
/* The plain per-call path: one request, blocking, on `stream`. */
int hyd_cuda_request_run(const hyd_request_t* req, void* stream);
/* Trace drivers with native timing: submit reqs[i] at t0 + arrival_s[i]
 * (seconds, ascending) and wait for all; latency_s[i] = arrival -> ready;
 * *elapsed_s = t0 -> last completion.  serve_trace uses the server; plain_trace
 * runs each request with hyd_cuda_request_run in arrival order. */
int hyd_cuda_serve_trace(hyd_server_t* srv, const hyd_request_t* reqs, const double* arrival_s, int64_t n,
                         double* latency_s, int* status, double* elapsed_s);
int hyd_cuda_plain_trace(const hyd_request_t* reqs, const double* arrival_s, int64_t n, double* latency_s,
                         int* status, double* elapsed_s, void* stream);

/* ---- host-memory entry points (embedding boundary) --------------------------
 * Same computations on HOST pointers: the input is streamed to the device in
 * 64 MiB chunks on two streams (copy of chunk k+1 overlaps the kernel on chunk
 * k) and the result read back.  Synchronous.  `hist` is overwritten with the
 * result of scatter (+) (fill [bins] 0) ... . */
int hyd_cuda_weighted_histogram_host(const int64_t* data, int64_t n, int64_t bins, int64_t* hist,
                                     int strategy);
int hyd_cuda_dot_f64_host(const double* xs, const double* ys, int64_t n, double* out);

/* Host array allocation compatible with the reference's hyd_array_free
 * (runtime/hydrangea_runtime.h:292-343): malloc'd header and storage record,
 * calloc'd data, refcount 1.  NULL on allocation failure. */
hyd_array_t* hyd_cuda_array_alloc(hyd_tuple_t shape, size_t elem_size);

/* Exported program symbols in the reference's export ABI (CodegenC.hs:
 * 372-460: `RET hyd_export_<name>(PARAMS)`), for the benchmark programs with
 * their inputs as parameters.  Like the reference's generated code they print
 * a message and exit(1) on failure (runtime/hydrangea_runtime.h:322-328).
 * Returned arrays are owned by the caller (free with hyd_array_free). */
hyd_array_t* hyd_export_weighted_histogram(hyd_array_t* data, int64_t bins);
/* demo/gray_scott's procedure (gray_scott.hyd:80; demo/gray_scott/main.cpp:85
 * calls it): V after 5000 steps on the demo's 256 x 256 grid from its initial
 * fields.  Memoised like the reference's zero-argument array procedures
 * (CodegenC.hs:812-833): computed on the first call; every call returns a view
 * over the same storage (reference count raised), freed with hyd_array_free.
 * hyd_cuda_cleanup drops the runtime's own reference. */
hyd_array_t* hyd_export_gray_scott(void);
/* The exports below read an input array from its device-resident copy when
 * the array is attached (next section); otherwise they stream its host data. */
double hyd_export_dot(hyd_array_t* xs, hyd_array_t* ys);

/* ---- runtime calls of generated host code -----------------------------------
 * What host code generated for `--backend cuda` calls around the device
 * primitives, in place of the reference runtime's helpers that the C backend's
 * generated code calls (runtime/hydrangea_runtime.h: array allocation and
 * release :292-343, hyd_get_env_int :602-616, the printers that main applies
 * to each zero-argument procedure :460-536).  They keep the reference's
 * behaviour: the printers write the same bytes, and a failure is a message on
 * stderr and exit(1), never a status.  Device work is ordered on the legacy
 * default stream.
 *   gen_check      exit(1) with the runtime's message unless status == 0
 *   gen_alloc      a device buffer (>= 1 byte); gen_free releases it
 *   gen_zero       zero `bytes` of a device buffer (the `fill [n] 0` of a scatter)
 *   gen_upload     a new device copy of a host array's data
 *   gen_download   a new host array (reference layout, refcount 1) of `shape`
 *                  from a device buffer, after reporting device-detected errors
 *   gen_read_*     one device scalar, after the same check
 *   gen_array_free the reference's hyd_array_free
 *   gen_get_env_int, gen_print_*: the reference's get_env_int and printers */
void hyd_cuda_gen_check(int status, const char* what);
void* hyd_cuda_gen_alloc(int64_t bytes);
void hyd_cuda_gen_free(void* d);
void hyd_cuda_gen_zero(void* d, int64_t bytes);
void* hyd_cuda_gen_upload(const hyd_array_t* a);
hyd_array_t* hyd_cuda_gen_download(const void* d, hyd_tuple_t shape, size_t elem_size);
int64_t hyd_cuda_gen_read_i64(const int64_t* d);
double hyd_cuda_gen_read_f64(const double* d);
void hyd_cuda_gen_array_free(hyd_array_t* a);
int64_t hyd_cuda_gen_get_env_int(const char* name);
void hyd_cuda_gen_print_int(int64_t v);
void hyd_cuda_gen_print_double(double v);
void hyd_cuda_gen_print_array(const hyd_array_t* a);
void hyd_cuda_gen_print_float_array(const hyd_array_t* a);

/* ---- the host I/O path: CSV files ------------------------------------------
 * Drop-in forms of the reference runtime's readers and writers
 * (hyd_read_array_csv / hyd_read_float_array_csv,
 * runtime/hydrangea_runtime.h:549-592; hyd_write_array_csv[_float],
 * runtime/hyd_write_csv.c): the same grammar, values, output bytes and
 * failures (a message on stderr, exit(1)), with the parsing and formatting
 * spread over all host threads.  The *_to_device / *_from_device forms parse
 * into pinned memory and copy to the device (or back) and return a status
 * instead of exiting. */
hyd_array_t* hyd_cuda_read_array_csv(const char* filename, hyd_tuple_t shape);
hyd_array_t* hyd_cuda_read_float_array_csv(const char* filename, hyd_tuple_t shape);
int64_t hyd_cuda_write_array_csv(hyd_array_t* arr, const char* filename);
int64_t hyd_cuda_write_array_csv_float(hyd_array_t* arr, const char* filename);
int hyd_cuda_read_csv_i64_to_device(const char* filename, int64_t n, int64_t* dev, void* stream);
int hyd_cuda_read_csv_f64_to_device(const char* filename, int64_t n, double* dev, void* stream);
int hyd_cuda_write_csv_i64_from_device(const int64_t* dev, hyd_tuple_t shape, const char* filename, void* stream);
int hyd_cuda_write_csv_f64_from_device(const double* dev, hyd_tuple_t shape, const char* filename, void* stream);

/* ---- device-resident arrays for the export path ----------------------------
 * The reference keeps arrays in host memory; its Metal export lifecycle keeps
 * the zero-argument array bindings as persistent GPU buffers across calls
 * (CodegenMSL.hs:1253-1300).  Here any host array can be made resident:
 *   attach         uploads the array and keeps a device copy beside
 *                  storage->data (valid until the host declares a write);
 *   host_modified  the host changed the data: the next use uploads again;
 *   device_data    the device copy (uploaded first if stale), NULL when the
 *                  array is not attached;
 *   detach         frees the copy; call it before hyd_array_free.
 * A copy belongs to (storage, data pointer, byte size): a view of another
 * extent is a separate array.  hyd_cuda_cleanup frees every copy.
 * resident_stats: attached arrays, uploads so far, resident bytes. */
int hyd_cuda_array_attach(hyd_array_t* a);
int hyd_cuda_array_host_modified(hyd_array_t* a);
int hyd_cuda_array_detach(hyd_array_t* a);
const void* hyd_cuda_array_device_data(hyd_array_t* a);
int hyd_cuda_array_resident_stats(int64_t* entries, int64_t* uploads, int64_t* bytes);

#ifdef __cplusplus
}
#endif
#endif /* HYD_CUDA_H */
