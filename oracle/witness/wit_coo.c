/* Witness: bench/coo_csr_build/coo_csr_build_ref.c (generate triplets, sort by
 * packed key, merge duplicates, row_ptr by prefix scan).  Copies the canonical
 * entries and row_ptr out and returns the canonical count.
 * TEST INFRASTRUCTURE ONLY. */
#define main wit_coo_unused_main
#include "bench/coo_csr_build/coo_csr_build_ref.c"
#undef main
int64_t wit_coo_csr(int64_t nrows, int64_t ncols, int64_t nnz, int64_t dup,
                    int64_t* row_ptr, int64_t* canon_rows, int64_t* canon_cols,
                    int64_t* canon_vals) {
    CooEntry* entries = (CooEntry*)malloc((size_t)nnz * sizeof(CooEntry));
    CooEntry* canonical = (CooEntry*)malloc((size_t)nnz * sizeof(CooEntry));
    CooData d = { nrows, ncols, nnz, dup, entries, canonical, row_ptr };
    (void)coo_run_once(&d);
    int64_t count = 0;
    for (int64_t i = 0; i < nnz; i++) {
        if (count == 0 || entries[i].packed_key != canonical[count - 1].packed_key) count++;
    }
    for (int64_t i = 0; i < count; i++) {
        canon_rows[i] = canonical[i].row;
        canon_cols[i] = canonical[i].col;
        canon_vals[i] = canonical[i].val;
    }
    free(entries);
    free(canonical);
    return count;
}
