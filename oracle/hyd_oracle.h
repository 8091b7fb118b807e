/* oracle/hyd_oracle.h -- CPU oracle for the Hydrangea fused-loop hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C99 + OpenMP,
 * the loop shapes that the reference C backend emits for the hot-path
 * combinators.  It is the checker for the CUDA runtime: only the test suite,
 * the smoke check and the CPU-baseline leg of bench.py may load it.  The
 * product (libhyd_cuda.so) never links or calls it.
 *
 * Each function names the reference file:line whose emitted loop it follows
 * (paths relative to the hydrangea-compiler source tree).
 */
#ifndef HYD_ORACLE_H
#define HYD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- seeded counter-based generators (shared bit-for-bit with the GPU) --- */
uint64_t orc_rand_u64(uint64_t seed, uint64_t i);
void orc_fill_uniform_f64(double* out, int64_t n, uint64_t seed, double lo, double hi);
void orc_fill_uniform_i64(int64_t* out, int64_t n, uint64_t seed, int64_t bound);

/* ---- reduce (+) 0.0 (zipwith (*) xs ys) -------------------------------- */
double orc_dot_f64(const double* xs, const double* ys, int64_t n);
double orc_dot_f64_serial(const double* xs, const double* ys, int64_t n);
double orc_dot_f64_compensated(const double* xs, const double* ys, int64_t n);
double orc_sum_f64_compensated(const double* xs, int64_t n);

/* ---- fused element chains (map / zipwith / generate) -------------------- */
void orc_map_chain_f64(int64_t n, double* out);
double orc_map_chain_sum_f64(int64_t n);
void orc_zipwith_muladd_f64(const double* a, const double* b, const double* c, double* out, int64_t n);

/* ---- scatter (+) ---------------------------------------------------------- */
int orc_weighted_hist_i64(const int64_t* data, int64_t n, int64_t bins, int64_t* hist);
int orc_weighted_hist_i64_atomic(const int64_t* data, int64_t n, int64_t bins, int64_t* hist);
int orc_hist_generate_i64(int64_t n, int64_t bins, int64_t* hist);
int orc_scatter_add_i64(const int64_t* idx, const int64_t* vals, int64_t n,
                        int64_t* dst, int64_t dst_n);
int orc_scatter_add_f64(const int64_t* idx, const double* vals, int64_t n,
                        double* dst, int64_t dst_n);

/* ---- stencils ------------------------------------------------------------- */
enum {
    ORC_ST_LAPLACIAN = 0,   /* a+b+c+d+(e*-4.0)               stencil_2d.hyd      */
    ORC_ST_JACOBI = 1,      /* (a+b+c+d)/4.0                  jacobi_2d.hyd       */
    ORC_ST_HEAT = 2,        /* e+0.1*((a+b+c+d)-(4.0*e))      heat step, 8192^2   */
    ORC_ST_HEAT_EXAMPLE = 3 /* (a+b+c+d+e)/5.0                examples/heat_2d.hyd */
};
void orc_stencil2d_f64(int kind, const double* in, double* out, int64_t h, int64_t w);
int orc_iterate_stencil2d_f64(int kind, double* buf0, double* buf1, int64_t h, int64_t w,
                              int64_t iters);
void orc_stencil1d_box3_i64(const int64_t* in, int64_t* out, int64_t n);
void orc_reduce_rows_i64(const int64_t* in, int64_t rows, int64_t cols, int op, int64_t init, int64_t* out);
void orc_reduce_rows_f64(const double* in, int64_t rows, int64_t cols, int op, double init, double* out);
int orc_scatter_add_guarded_i64(const int64_t* idx, const int64_t* vals, const int64_t* guard, int64_t n,
                                int64_t* dst, int64_t dst_n);
/* boundary conditions (Syntax.hs:416-426; index arithmetic Lowering.hs:2762-2870) */
enum { ORC_BND_CLAMP = 0, ORC_BND_WRAP = 1, ORC_BND_MIRROR = 2, ORC_BND_CONST = 3 };
int64_t orc_bound_index(int64_t raw, int64_t n, int mode);
int orc_stencil1d_offsets_i64(const int64_t* in, int64_t* out, int64_t n, const int64_t* offs, int noff,
                              int mode, int64_t fill);
int orc_stencil2d_offsets_i64(const int64_t* in, int64_t* out, int64_t h, int64_t w, const int64_t* offs,
                              int noff, int mode, int64_t fill);
int orc_stencil2d_bnd_f64(int kind, int mode, double fill, const double* in, double* out, int64_t h,
                          int64_t w);
int orc_iterate_stencil2d_bnd_f64(int kind, int mode, double fill, double* buf0, double* buf1, int64_t h,
                                  int64_t w, int64_t iters);
void orc_stencil1d_jacobi3_f64(const double* in, double* out, int64_t n);
int orc_iterate_stencil1d_jacobi3_f64(double* buf0, double* buf1, int64_t n, int64_t iters);
void orc_gray_scott_step_f64(const double* u, const double* v, double* un, double* vn, int64_t h, int64_t w,
                             double du, double dv, double feed, double kill, double dt);

/* ---- scan family and segmented reduce ------------------------------------ */
void orc_scan_i64(const int64_t* in, int64_t* out, int64_t n, int64_t init,
                  int reverse, int inclusive);
void orc_scan_f64(const double* in, double* out, int64_t n, double init,
                  int reverse, int inclusive);
int orc_segmented_reduce_i64(const int64_t* offsets, int64_t n_offsets,
                             const int64_t* vals, int64_t n_vals, int64_t init,
                             int64_t* out);
int orc_segmented_reduce_f64(const int64_t* offsets, int64_t n_offsets,
                             const double* vals, int64_t n_vals, double init,
                             double* out);

/* ---- sort / gather / COO / CSR / SpMV -------------------------------------- */
void orc_sort_indices_i64(const int64_t* keys, int64_t n, int64_t* perm);
void orc_gather_i64(const int64_t* perm, int64_t n, const int64_t* src, int64_t* out);
void orc_gather_f64(const int64_t* perm, int64_t n, const double* src, double* out);
int64_t orc_coo_sum_duplicates_i64(const int64_t* rows, const int64_t* cols,
                                   const int64_t* vals, int64_t nnz,
                                   int64_t* out_rows, int64_t* out_cols, int64_t* out_vals);
int orc_csr_from_sorted_coo_i64(int64_t nrows, int64_t nnz, const int64_t* rows,
                                const int64_t* cols, const int64_t* vals,
                                int64_t* row_ptr, int64_t* col_idx, int64_t* out_vals);
void orc_spmv_csr_f64(int64_t nrows, const int64_t* row_ptr, const int64_t* col_idx,
                      const double* vals, const double* x, double* y);
int orc_coo_to_csr_spmv_f64(int64_t nrows, int64_t ncols, int64_t nnz,
                            const int32_t* rows, const int32_t* cols, const double* vals,
                            const double* x, int64_t* row_ptr, int32_t* col_idx,
                            double* csr_vals, double* y);
void orc_coo_csr_bench_inputs(int64_t nrows, int64_t ncols, int64_t nnz, int64_t dup,
                              int64_t* rows, int64_t* cols, int64_t* vals);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
