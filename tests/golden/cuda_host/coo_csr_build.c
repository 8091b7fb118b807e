/* Host program of the --backend cuda path for bench/coo_csr_build/coo_csr_build.hyd, emitted by codegen_cuda.py.
 * Each fused loop nest is one call into the GB300 runtime (libhyd_cuda.so);
 * procedures return the reference runtime's host arrays. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "hyd_cuda.h"

static int64_t nrows(void) {
    int64_t v = hyd_cuda_gen_get_env_int("COO_NROWS");
    return v;
}

static int64_t ncols(void) {
    int64_t v = hyd_cuda_gen_get_env_int("COO_NCOLS");
    return v;
}

static int64_t nnz(void) {
    int64_t v = hyd_cuda_gen_get_env_int("COO_NNZ");
    return v;
}

static int64_t dup(void) {
    int64_t v = hyd_cuda_gen_get_env_int("COO_DUP_PERIOD");
    return v;
}

static int64_t imod(int64_t x, int64_t m) {
    return x - ((x / m) * m);
}

static int64_t hyd_main(void) {
    int64_t nr = nrows();
    int64_t nc = ncols();
    int64_t nz = nnz();
    int64_t dp = dup();
    int64_t* d_rows = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    {
        char body[512];
        snprintf(body, sizeof body, "long long g = i / %lldLL; long long a = g * 17 + 3; v = a - ((a / %lldLL) * %lldLL);", (long long)dp, (long long)nr, (long long)nr);
        hyd_cuda_gen_check(hyd_cuda_map_i64(body, NULL, 0, nz, d_rows, NULL, NULL), "map_i64");
    }
    int64_t* d_cols = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    {
        char body[512];
        snprintf(body, sizeof body, "long long g = i / %lldLL; long long a = g * 31 + 7; v = a - ((a / %lldLL) * %lldLL);", (long long)dp, (long long)nc, (long long)nc);
        hyd_cuda_gen_check(hyd_cuda_map_i64(body, NULL, 0, nz, d_cols, NULL, NULL), "map_i64");
    }
    int64_t* d_vals = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    {
        char body[512];
        snprintf(body, sizeof body, "long long g = i / %lldLL; v = (g * 13) + i + 1;", (long long)dp);
        hyd_cuda_gen_check(hyd_cuda_map_i64(body, NULL, 0, nz, d_vals, NULL, NULL), "map_i64");
    }
    int64_t* d_keys = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    {
        char body[512];
        snprintf(body, sizeof body, "long long g = i / %lldLL; long long a = g * 17 + 3; long long b = g * 31 + 7; v = (a - ((a / %lldLL) * %lldLL)) * %lldLL + (b - ((b / %lldLL) * %lldLL));", (long long)dp, (long long)nr, (long long)nr, (long long)nc, (long long)nc, (long long)nc);
        hyd_cuda_gen_check(hyd_cuda_map_i64(body, NULL, 0, nz, d_keys, NULL, NULL), "map_i64");
    }
    int64_t* d_perm = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    hyd_cuda_gen_check(hyd_cuda_sort_indices_i64(d_keys, nz, d_perm, NULL), "sort_indices");
    int64_t* d_srows = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    hyd_cuda_gen_check(hyd_cuda_gather_i64(d_perm, nz, d_rows, nz, d_srows, NULL), "gather");
    int64_t* d_scols = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    hyd_cuda_gen_check(hyd_cuda_gather_i64(d_perm, nz, d_cols, nz, d_scols, NULL), "gather");
    int64_t* d_svals = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    hyd_cuda_gen_check(hyd_cuda_gather_i64(d_perm, nz, d_vals, nz, d_svals, NULL), "gather");
    int64_t* d_crows = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    int64_t* d_ccols = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    int64_t* d_cvals = (int64_t*)hyd_cuda_gen_alloc((nz) * (int64_t)sizeof(int64_t));
    int64_t cnnz;
    {
        int64_t* cnt = (int64_t*)hyd_cuda_gen_alloc((int64_t)sizeof(int64_t));
        hyd_cuda_gen_check(hyd_cuda_coo_sum_duplicates_i64(d_srows, d_scols, d_svals, nz, d_crows, d_ccols, d_cvals, cnt, NULL), "coo_sum_duplicates");
        cnnz = hyd_cuda_gen_read_i64(cnt);
        hyd_cuda_gen_free(cnt);
    }
    int64_t* d_row_ptr = (int64_t*)hyd_cuda_gen_alloc((nr + 1) * (int64_t)sizeof(int64_t));
    int64_t* d_col_idx = (int64_t*)hyd_cuda_gen_alloc((cnnz) * (int64_t)sizeof(int64_t));
    int64_t* d_csr_vals = (int64_t*)hyd_cuda_gen_alloc((cnnz) * (int64_t)sizeof(int64_t));
    hyd_cuda_gen_check(hyd_cuda_csr_from_sorted_coo_i64(nr, cnnz, d_crows, d_ccols, d_cvals, d_row_ptr, d_col_idx, d_csr_vals, NULL), "csr_from_sorted_coo");
    int64_t s_row_ptr;
    {
        int64_t* acc = (int64_t*)hyd_cuda_gen_alloc((int64_t)sizeof(int64_t));
        const int64_t* in[1] = {d_row_ptr};
        hyd_cuda_gen_check(hyd_cuda_map_i64("v = x0;", in, 1, nr + 1, NULL, acc, NULL), "reduce (+)");
        s_row_ptr = hyd_cuda_gen_read_i64(acc);
        hyd_cuda_gen_free(acc);
    }
    int64_t s_col_idx;
    {
        int64_t* acc = (int64_t*)hyd_cuda_gen_alloc((int64_t)sizeof(int64_t));
        const int64_t* in[1] = {d_col_idx};
        hyd_cuda_gen_check(hyd_cuda_map_i64("v = x0;", in, 1, cnnz, NULL, acc, NULL), "reduce (+)");
        s_col_idx = hyd_cuda_gen_read_i64(acc);
        hyd_cuda_gen_free(acc);
    }
    int64_t s_vals;
    {
        int64_t* acc = (int64_t*)hyd_cuda_gen_alloc((int64_t)sizeof(int64_t));
        const int64_t* in[1] = {d_csr_vals};
        hyd_cuda_gen_check(hyd_cuda_map_i64("v = x0;", in, 1, cnnz, NULL, acc, NULL), "reduce (+)");
        s_vals = hyd_cuda_gen_read_i64(acc);
        hyd_cuda_gen_free(acc);
    }
    int64_t checksum = s_row_ptr + s_col_idx + s_vals + cnnz;
    hyd_cuda_gen_free(d_rows);
    hyd_cuda_gen_free(d_cols);
    hyd_cuda_gen_free(d_vals);
    hyd_cuda_gen_free(d_keys);
    hyd_cuda_gen_free(d_perm);
    hyd_cuda_gen_free(d_srows);
    hyd_cuda_gen_free(d_scols);
    hyd_cuda_gen_free(d_svals);
    hyd_cuda_gen_free(d_crows);
    hyd_cuda_gen_free(d_ccols);
    hyd_cuda_gen_free(d_cvals);
    hyd_cuda_gen_free(d_row_ptr);
    hyd_cuda_gen_free(d_col_idx);
    hyd_cuda_gen_free(d_csr_vals);
    return checksum;
}

int64_t hyd_export_imod(int64_t x, int64_t m) {
    return imod(x, m);
}

int main(void) {
    hyd_cuda_gen_check(hyd_cuda_init(), "hyd_cuda_init");
    int64_t nrows_result = nrows();
    hyd_cuda_gen_print_int(nrows_result);
    int64_t ncols_result = ncols();
    hyd_cuda_gen_print_int(ncols_result);
    int64_t nnz_result = nnz();
    hyd_cuda_gen_print_int(nnz_result);
    int64_t dup_result = dup();
    hyd_cuda_gen_print_int(dup_result);
    int64_t hyd_main_result = hyd_main();
    hyd_cuda_gen_print_int(hyd_main_result);
    hyd_cuda_cleanup();
    return 0;
}
