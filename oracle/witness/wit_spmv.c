/* Witness: bench/spmv/spmv_ref.c (OpenMP CSR SpMV). TEST INFRASTRUCTURE ONLY. */
#define main wit_spmv_unused_main
#include "bench/spmv/spmv_ref.c"
#undef main
void wit_spmv(int64_t nrows, int64_t ncols, int64_t nnz, double* values, int64_t* col_idx,
              int64_t* row_ptr, double* x, double* y) {
    SPMVData d = { nrows, ncols, nnz, values, col_idx, row_ptr, x, y };
    (void)spmv_run_once(&d);
}
