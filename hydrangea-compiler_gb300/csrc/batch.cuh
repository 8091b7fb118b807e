// batch.cuh -- the batched COO -> CSR -> SpMV pipeline's instance descriptor,
// shared by sparse.cu (the pipeline) and serve.cu (which coalesces SpMV
// requests into it).
#pragma once

#include <vector>

#include "hyd_common.cuh"

namespace hyd {

// Instance descriptor (device table).  Every instance has its own arrays;
// counts/row_start are batch-wide scratch indexed by row_base + row, and the
// batch-wide exclusive scan of the counts reaches scan_base (= entries of all
// earlier instances) at the instance's first row.
struct BatchInst {
    long long nrows, ncols, nnz;
    long long row_base;   // first row of this instance in the batch-wide row space
    long long scan_base;  // entries of all earlier instances
    const int* rows;
    const int* cols;
    const double* vals;
    const double* x;
    long long* row_ptr;   // nrows + 1
    int* csr_cols;
    double* csr_vals;
    double* y;
};

// Runs count -> scan -> scatter -> sort+SpMV for `inst` (see sparse.cu).
int batch_pipeline(std::vector<BatchInst>& inst, const char* key, cudaStream_t s, void* staging,
                   size_t staging_bytes);
size_t batch_pipeline_table_bytes(const std::vector<BatchInst>& inst);

}  // namespace hyd
