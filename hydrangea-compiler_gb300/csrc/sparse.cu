// sparse.cu -- coo_sum_duplicates, csr_from_sorted_coo, CSR SpMV, and the
// batched COO -> CSR -> SpMV pipeline over many instances of uneven size.
//
// Reference: coo_sum_duplicates (Lowering.hs:966-1080) merges adjacent equal
// (row, col) entries in one serial pass; csr_from_sorted_coo
// (Lowering.hs:1081-1160) counts entries per row, copies cols/vals through and
// turns the counts into row_ptr with a serial running sum; SpMV is the
// generate-of-reduce_generate of bench/spmv/spmv.hyd:30-40 (outer loop over
// rows in `omp parallel for`, sequential sum per row).
//
// GPU forms:
//  * coo_sum_duplicates: head flags -> inclusive scan (segment ids) -> heads
//    write (row, col), every entry adds its value into its segment (int64,
//    order-independent, bit-exact); entries past the canonical count are
//    zeroed like the reference's calloc'd outputs.
//  * csr_from_sorted_coo: row counts by global atomics, exclusive scan
//    (decoupled look-back), parallel copy of cols/vals.
//  * SpMV: a group of G lanes per row (G from the average row length: the
//    vector width the autotuner chooses), lane-strided fma partial sums and a
//    fixed xor tree, so results are deterministic; within 1e-12 of
//    sum |v*x| of the C backend's sequential sum.
//  * batched pipeline: instances are described by a device table; persistent
//    CTAs drain a device-side queue of (instance, tile) work items through an
//    atomic cursor, so one launch covers 512 instances of 10^3..10^6 entries
//    with no per-instance launch.  Stages: (1) count entries per global row,
//    (2) one exclusive scan over all instances' rows gives every row's first
//    slot (instance ranges are contiguous, so this is also each instance's
//    row_ptr shifted by its entry base), (3) scatter every entry into its row
//    (atomic slot within the row), (4) per row: sort by column and compute that
//    row's SpMV (one fma chain in column order) in the same warp.  Columns are unique within a row in this
//    workload, so sorting fixes the in-row order and the CSR is bit-exact
//    however the atomics interleaved.
#include <cstdlib>
#include <cstring>
#include <vector>

#include "batch.cuh"
#include "hyd_common.cuh"

namespace hyd {

int scan_i64_launch(const long long* in, long long* out, int64_t n, long long init, bool reverse,
                    bool inclusive, cudaStream_t stream);

// ---------------------------------------------------------------- coo dedup
__global__ void coo_head_flags_kernel(const long long* __restrict__ rows, const long long* __restrict__ cols,
                                      int64_t nnz, long long* __restrict__ flags) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x)
        flags[i] = (i == 0 || rows[i] != rows[i - 1] || cols[i] != cols[i - 1]) ? 1 : 0;
}

__global__ void coo_merge_kernel(const long long* __restrict__ rows, const long long* __restrict__ cols,
                                 const long long* __restrict__ vals, int64_t nnz,
                                 const long long* __restrict__ seg_incl, long long* __restrict__ out_rows,
                                 long long* __restrict__ out_cols, unsigned long long* __restrict__ out_vals) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const long long s = seg_incl[i] - 1;
        const bool head = (i == 0) || seg_incl[i] != seg_incl[i - 1];
        if (head) {
            out_rows[s] = rows[i];
            out_cols[s] = cols[i];
        }
        atomicAdd(&out_vals[s], (unsigned long long)vals[i]);
    }
}

// ---------------------------------------------------------------- csr build
__global__ void csr_count_kernel(const long long* __restrict__ rows, int64_t nnz, int64_t nrows,
                                 unsigned long long* __restrict__ counts, unsigned* err) {
    bool bad = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const long long r = rows[i];
        if ((unsigned long long)r < (unsigned long long)nrows) atomicAdd(&counts[r], 1ULL);
        else bad = true;
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

template <class T>
__global__ void copy_kernel(const T* __restrict__ src, T* __restrict__ dst, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

__global__ void set_last_kernel(long long* row_ptr, int64_t nrows, const long long* scan_in, const long long* scan_out) {
    // row_ptr[nrows] = total = exclusive prefix of the last row + its count
    if (threadIdx.x == 0 && blockIdx.x == 0)
        row_ptr[nrows] = nrows > 0 ? scan_out[nrows - 1] + scan_in[nrows - 1] : 0;
}

// ---------------------------------------------------------------- SpMV
template <int G, class C>
__global__ void __launch_bounds__(256) spmv_csr_kernel(int64_t nrows, const long long* __restrict__ row_ptr,
                                                       const C* __restrict__ col_idx,
                                                       const double* __restrict__ vals,
                                                       const double* __restrict__ x, int64_t ncols,
                                                       double* __restrict__ y, unsigned* err) {
    const int sub = threadIdx.x & (G - 1);
    constexpr int kRowsPerWarp = 32 / G;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int group = (threadIdx.x & 31) / G;
    bool bad = false;
    // warp-uniform loop: every lane of a warp runs the same iterations, so the
    // full-mask shuffles below always see all 32 lanes
    for (int64_t rb = warp * kRowsPerWarp; rb < nrows; rb += warps * kRowsPerWarp) {
        const int64_t r = rb + group;
        double acc = 0.0;
        if (r < nrows) {
            const long long s = row_ptr[r], e = row_ptr[r + 1];
            for (long long k = s + sub; k < e; k += G) {
                const long long c = (long long)col_idx[k];
                if ((unsigned long long)c < (unsigned long long)ncols) acc = fma(vals[k], x[c], acc);
                else bad = true;
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (sub == 0 && r < nrows) y[r] = acc;
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

template <class C>
static int spmv_dispatch(int g, int64_t nrows, const long long* row_ptr, const C* col_idx, const double* vals,
                         const double* x, int64_t ncols, double* y, const Device* d, cudaStream_t stream) {
    int64_t blocks = (nrows * g + 255) / 256;
    const int64_t cap = (int64_t)d->sm_count * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    switch (g) {
        case 1: spmv_csr_kernel<1, C><<<(unsigned)blocks, 256, 0, stream>>>(nrows, row_ptr, col_idx, vals, x, ncols, y, d->d_err); break;
        case 2: spmv_csr_kernel<2, C><<<(unsigned)blocks, 256, 0, stream>>>(nrows, row_ptr, col_idx, vals, x, ncols, y, d->d_err); break;
        case 4: spmv_csr_kernel<4, C><<<(unsigned)blocks, 256, 0, stream>>>(nrows, row_ptr, col_idx, vals, x, ncols, y, d->d_err); break;
        case 8: spmv_csr_kernel<8, C><<<(unsigned)blocks, 256, 0, stream>>>(nrows, row_ptr, col_idx, vals, x, ncols, y, d->d_err); break;
        case 16: spmv_csr_kernel<16, C><<<(unsigned)blocks, 256, 0, stream>>>(nrows, row_ptr, col_idx, vals, x, ncols, y, d->d_err); break;
        default: spmv_csr_kernel<32, C><<<(unsigned)blocks, 256, 0, stream>>>(nrows, row_ptr, col_idx, vals, x, ncols, y, d->d_err); break;
    }
    return launch_check("spmv_csr");
}

// ---------------------------------------------------------------- batched pipeline
struct WorkItem {
    int inst;
    int tile;  // tile index inside the instance
};

constexpr int kBatchThreads = 256;
constexpr int kEntryTile = 8192;  // entries per work item (count and scatter stages)
constexpr int kRowTile = 256;     // rows per work item (sort + SpMV stage): one warp per row

__device__ __forceinline__ bool next_item(unsigned* cursor, unsigned nitems, unsigned& item) {
    __shared__ unsigned sh_item;
    if (threadIdx.x == 0) sh_item = atomicAdd(cursor, 1u);
    __syncthreads();
    item = sh_item;
    __syncthreads();
    return item < nitems;
}

// Stage 1: row counts (and validation of every entry).
__global__ void __launch_bounds__(kBatchThreads) batch_count_kernel(const BatchInst* __restrict__ inst,
                                                                    const WorkItem* __restrict__ items, unsigned nitems,
                                                                    unsigned* cursor, unsigned* __restrict__ counts,
                                                                    unsigned* err) {
    unsigned it;
    bool bad = false;
    while (next_item(cursor, nitems, it)) {
        const WorkItem w = items[it];
        const BatchInst I = inst[w.inst];
        const long long t0 = (long long)w.tile * kEntryTile;
        const long long t1 = t0 + kEntryTile < I.nnz ? t0 + kEntryTile : I.nnz;
        for (long long k = t0 + threadIdx.x; k < t1; k += kBatchThreads) {
            const int r = I.rows[k], c = I.cols[k];
            if (r >= 0 && r < I.nrows && c >= 0 && c < I.ncols) atomicAdd(&counts[I.row_base + r], 1u);
            else bad = true;
        }
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// Counts (u32) -> int64 for the scan.
__global__ void widen_kernel(const unsigned* __restrict__ c, long long* __restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = c[i];
}

// Stage 3: scatter entries to their row's slots (slot order within a row is
// arbitrary here; stage 4 sorts each row).  counts[] counts down to 0.
__global__ void __launch_bounds__(kBatchThreads) batch_scatter_kernel(const BatchInst* __restrict__ inst,
                                                                      const WorkItem* __restrict__ items,
                                                                      unsigned nitems, unsigned* cursor,
                                                                      const long long* __restrict__ row_start,
                                                                      unsigned* __restrict__ counts,
                                                                      unsigned* __restrict__ coo_idx) {
    unsigned it;
    while (next_item(cursor, nitems, it)) {
        const WorkItem w = items[it];
        const BatchInst I = inst[w.inst];
        const long long t0 = (long long)w.tile * kEntryTile;
        const long long t1 = t0 + kEntryTile < I.nnz ? t0 + kEntryTile : I.nnz;
        for (long long k = t0 + threadIdx.x; k < t1; k += kBatchThreads) {
            const int r = I.rows[k], c = I.cols[k];
            if (r < 0 || r >= I.nrows || c < 0 || c >= I.ncols) continue;  // reported by stage 1
            const long long g = I.row_base + r;
            const unsigned left = atomicSub(&counts[g], 1u);  // slots of row g still free
            const long long slot = row_start[g] - I.scan_base + (long long)left - 1;
            I.csr_cols[slot] = c;
            I.csr_vals[slot] = I.vals[k];
            coo_idx[I.scan_base + slot] = (unsigned)k;  // orders equal columns in stage 4
        }
    }
}

// Warp-wide bitonic sort of up to 32*kPer (key, val) pairs held kPer per lane
// in "lane-major" order (element j*32 + lane in slot j).  Padding uses the
// largest key.
template <int kPer, class K>
__device__ __forceinline__ void warp_bitonic_sort(K (&key)[kPer], double (&val)[kPer]) {
    const int lane = threadIdx.x & 31;
    constexpr int N = 32 * kPer;
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= 32) {
                // partner in another slot of the same lane
                const int sj = stride / 32;
#pragma unroll
                for (int j = 0; j < kPer; ++j) {
                    if ((j & sj) == 0) {
                        const int idx = j * 32 + lane;
                        const bool up = (idx & size) == 0;
                        const int jj = j + sj;
                        const bool swap = up ? (key[j] > key[jj]) : (key[j] < key[jj]);
                        if (swap) {
                            const K tk = key[j]; key[j] = key[jj]; key[jj] = tk;
                            double tv = val[j]; val[j] = val[jj]; val[jj] = tv;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < kPer; ++j) {
                    const int idx = j * 32 + lane;
                    const K ok = __shfl_xor_sync(0xffffffffu, key[j], stride);
                    const double ov = __shfl_xor_sync(0xffffffffu, val[j], stride);
                    const bool up = (idx & size) == 0;
                    const bool lower = (lane & stride) == 0;
                    // the lower index keeps the smaller key when ascending
                    const bool take = lower ? (up ? ok < key[j] : ok > key[j]) : (up ? ok > key[j] : ok < key[j]);
                    if (take) {
                        key[j] = ok;
                        val[j] = ov;
                    }
                }
            }
        }
    }
}

// Sort key: column, then COO position -- the runtime's stable order for equal
// (row, col) entries.
// Columns are bounded by ncols before x is read: with invalid entries in the
// batch (reported by stage 1) a row can include a slot that no entry wrote,
// and whatever it holds must not index x.
template <int kPer>
__device__ __forceinline__ void sort_row_and_spmv(int* __restrict__ cc, double* __restrict__ cv,
                                                  const unsigned* __restrict__ coo_idx, int len,
                                                  const double* __restrict__ x, long long ncols, double* yrow) {
    const int lane = threadIdx.x & 31;
    long long key[kPer];
    double val[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int i = j * 32 + lane;
        key[j] = i < len ? (((long long)cc[i] << 32) | coo_idx[i]) : 0x7fffffffffffffffLL;
        val[j] = i < len ? cv[i] : 0.0;
    }
    warp_bitonic_sort<kPer>(key, val);
    double xv[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int i = j * 32 + lane;
        xv[j] = 0.0;
        if (i < len) {
            const int c = (int)(key[j] >> 32);
            cc[i] = c;
            cv[i] = val[j];
            if ((unsigned)c < (unsigned long long)ncols) xv[j] = x[c];
        }
    }
    // y: one fma chain over the row in column order (position i sits on lane
    // i % 32, register i / 32), the order of the bucketed form
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        for (int l = 0; l < 32 && j * 32 + l < len; ++l)
            acc = fma(__shfl_sync(0xffffffffu, val[j], l), __shfl_sync(0xffffffffu, xv[j], l), acc);
    }
    if (lane == 0) *yrow = acc;
}

// Stage 4: per row (one warp): sort by column, write back, y[row] = sum v*x[c].
// Also writes the instance's row_ptr (relative to its entry base).
__global__ void __launch_bounds__(kBatchThreads) batch_sort_spmv_kernel(
    const BatchInst* __restrict__ inst, const WorkItem* __restrict__ items, unsigned nitems, unsigned* cursor,
    const long long* __restrict__ row_start, const unsigned* __restrict__ coo_idx, unsigned* err) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int W = kBatchThreads / 32;
    unsigned it;
    bool bad = false;
    while (next_item(cursor, nitems, it)) {
        const WorkItem w = items[it];
        const BatchInst I = inst[w.inst];
        const long long r0 = (long long)w.tile * kRowTile;
        const long long r1 = r0 + kRowTile < I.nrows ? r0 + kRowTile : I.nrows;
        for (long long r = r0 + warp; r < r1; r += W) {
            const long long g = I.row_base + r;
            long long s = row_start[g] - I.scan_base;
            long long e = (r + 1 < I.nrows) ? row_start[g + 1] - I.scan_base : I.nnz;
            // with invalid entries (reported by stage 1) the counts and the
            // instance's extent disagree: keep the span inside the instance
            s = s < 0 ? 0 : (s > I.nnz ? I.nnz : s);
            e = e < s ? s : (e > I.nnz ? I.nnz : e);
            const int len = (int)(e - s);
            if (lane == 0) {
                I.row_ptr[r] = s;
                if (r == I.nrows - 1) I.row_ptr[I.nrows] = I.nnz;
            }
            int* cc = I.csr_cols + s;
            double* cv = I.csr_vals + s;
            const unsigned* ci = coo_idx + I.scan_base + s;
            if (len <= 32) sort_row_and_spmv<1>(cc, cv, ci, len, I.x, I.ncols, I.y + r);
            else if (len <= 64) sort_row_and_spmv<2>(cc, cv, ci, len, I.x, I.ncols, I.y + r);
            else if (len <= 128) sort_row_and_spmv<4>(cc, cv, ci, len, I.x, I.ncols, I.y + r);
            else if (len <= 256) sort_row_and_spmv<8>(cc, cv, ci, len, I.x, I.ncols, I.y + r);
            else bad = true;  // rows above 256 entries are outside this kernel's contract
        }
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// Runs the four stages for a batch described by host-side `inst` (row_base and
// scan_base filled here).  Scratch comes from the named device buffer `key`.
// With `staging` (pinned host memory of `staging_bytes`, kept alive by the
// caller until the stream reaches this point) the tables are copied
// asynchronously and the call returns without synchronizing; otherwise it
// synchronizes the stream before returning.
// Row-atomic form (see the file comment); the fallback of the bucketed form.
int batch_pipeline_rows(std::vector<BatchInst>& inst, const char* key, cudaStream_t s, void* staging,
                        size_t staging_bytes) {
    Device* d = nullptr;
    HYD_TRY(device(&d));
    std::vector<WorkItem> count_items, row_items;
    long long rows_total = 0, entries = 0;
    for (size_t i = 0; i < inst.size(); ++i) {
        BatchInst& I = inst[i];
        I.row_base = rows_total;
        I.scan_base = entries;
        for (long long t = 0; t * kEntryTile < I.nnz; ++t) count_items.push_back(WorkItem{(int)i, (int)t});
        for (long long t = 0; t * kRowTile < I.nrows; ++t) row_items.push_back(WorkItem{(int)i, (int)t});
        rows_total += I.nrows;
        entries += I.nnz;
    }
    if (rows_total >= (1LL << 32)) return set_error(HYD_CUDA_ERR_UNSUPPORTED, "batch: too many rows");
    for (const BatchInst& I : inst)  // COO positions are kept as 32-bit indices
        if (I.nnz > (1LL << 32)) return set_error(HYD_CUDA_ERR_UNSUPPORTED, "batch: instance above 2^32 entries");
    const size_t inst_bytes = (inst.size() * sizeof(BatchInst) + 255) & ~(size_t)255;
    const size_t ci_bytes = ((count_items.size() * sizeof(WorkItem)) + 255) & ~(size_t)255;
    const size_t ri_bytes = ((row_items.size() * sizeof(WorkItem)) + 255) & ~(size_t)255;
    const size_t cnt_bytes = ((size_t)rows_total * 4 + 255) & ~(size_t)255;
    const size_t wide_bytes = ((size_t)rows_total * 8 + 255) & ~(size_t)255;
    void* buf = nullptr;
    const size_t idx_bytes = ((size_t)entries * 4 + 255) & ~(size_t)255;
    HYD_TRY(device_buffer(d, key, inst_bytes + ci_bytes + ri_bytes + cnt_bytes + 2 * wide_bytes + 256 + idx_bytes,
                          &buf));
    unsigned char* b = static_cast<unsigned char*>(buf);
    BatchInst* d_inst = reinterpret_cast<BatchInst*>(b);
    WorkItem* d_ci = reinterpret_cast<WorkItem*>(b + inst_bytes);
    WorkItem* d_ri = reinterpret_cast<WorkItem*>(b + inst_bytes + ci_bytes);
    unsigned* counts = reinterpret_cast<unsigned*>(b + inst_bytes + ci_bytes + ri_bytes);
    long long* wide = reinterpret_cast<long long*>(b + inst_bytes + ci_bytes + ri_bytes + cnt_bytes);
    long long* row_start = wide + (wide_bytes / 8);
    unsigned* cursors = reinterpret_cast<unsigned*>(b + inst_bytes + ci_bytes + ri_bytes + cnt_bytes + 2 * wide_bytes);
    unsigned* coo_idx = reinterpret_cast<unsigned*>(b + inst_bytes + ci_bytes + ri_bytes + cnt_bytes + 2 * wide_bytes + 256);
    const size_t table_bytes = inst_bytes + ci_bytes + ri_bytes;
    const unsigned char* src_inst = reinterpret_cast<const unsigned char*>(inst.data());
    const unsigned char* src_ci = reinterpret_cast<const unsigned char*>(count_items.data());
    const unsigned char* src_ri = reinterpret_cast<const unsigned char*>(row_items.data());
    const bool async_tables = staging != nullptr && staging_bytes >= table_bytes;
    if (async_tables) {
        unsigned char* h = static_cast<unsigned char*>(staging);
        memcpy(h, src_inst, inst.size() * sizeof(BatchInst));
        if (!count_items.empty()) memcpy(h + inst_bytes, src_ci, count_items.size() * sizeof(WorkItem));
        memcpy(h + inst_bytes + ci_bytes, src_ri, row_items.size() * sizeof(WorkItem));
        HYD_CUDA_TRY(cudaMemcpyAsync(b, h, table_bytes, cudaMemcpyHostToDevice, s));
    } else {
        HYD_CUDA_TRY(cudaMemcpyAsync(d_inst, src_inst, inst.size() * sizeof(BatchInst), cudaMemcpyHostToDevice, s));
        if (!count_items.empty())
            HYD_CUDA_TRY(cudaMemcpyAsync(d_ci, src_ci, count_items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, s));
        HYD_CUDA_TRY(cudaMemcpyAsync(d_ri, src_ri, row_items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, s));
    }
    HYD_CUDA_TRY(cudaMemsetAsync(counts, 0, (size_t)rows_total * 4, s));
    HYD_CUDA_TRY(cudaMemsetAsync(cursors, 0, 16, s));
    const unsigned grid = (unsigned)(d->sm_count * 8);
    if (!count_items.empty()) {
        batch_count_kernel<<<grid, kBatchThreads, 0, s>>>(d_inst, d_ci, (unsigned)count_items.size(), cursors + 0,
                                                          counts, d->d_err);
        HYD_TRY(launch_check("batch_count"));
    }
    widen_kernel<<<grid, 256, 0, s>>>(counts, wide, rows_total);
    HYD_TRY(launch_check("batch_widen"));
    HYD_TRY(scan_i64_launch(wide, row_start, rows_total, 0, false, false, s));
    if (!count_items.empty()) {
        batch_scatter_kernel<<<grid, kBatchThreads, 0, s>>>(d_inst, d_ci, (unsigned)count_items.size(), cursors + 1,
                                                            row_start, counts, coo_idx);
        HYD_TRY(launch_check("batch_scatter"));
    }
    batch_sort_spmv_kernel<<<grid, kBatchThreads, 0, s>>>(d_inst, d_ri, (unsigned)row_items.size(), cursors + 2,
                                                          row_start, coo_idx, d->d_err);
    HYD_TRY(launch_check("batch_sort_spmv"));
    // pageable tables die with the caller's vectors: the copies must have run
    if (!async_tables) HYD_CUDA_TRY(cudaStreamSynchronize(s));
    return HYD_CUDA_OK;
}

int batch_pipeline_bucketed(std::vector<BatchInst>& bi, const char* key, cudaStream_t s, void* staging,
                            size_t staging_bytes);
size_t batch_pipeline_bucketed_table_bytes(const std::vector<BatchInst>& bi);

// The batched pipeline: the bucketed form (sparse_bucket.cu) when the batch is
// within its limits, otherwise the row-atomic form.
int batch_pipeline(std::vector<BatchInst>& inst, const char* key, cudaStream_t s, void* staging,
                   size_t staging_bytes) {
    const char* force = getenv("HYD_CUDA_BATCH_PIPELINE");  // "rows" forces the row-atomic form
    if (!(force && strcmp(force, "rows") == 0)) {
        const int st = batch_pipeline_bucketed(inst, key, s, staging, staging_bytes);
        if (st != HYD_CUDA_ERR_UNSUPPORTED) return st;
    }
    return batch_pipeline_rows(inst, key, s, staging, staging_bytes);
}

static size_t batch_pipeline_rows_table_bytes(const std::vector<BatchInst>& inst);

// Bytes of pinned staging batch_pipeline needs for `inst`.
size_t batch_pipeline_table_bytes(const std::vector<BatchInst>& inst) {
    const size_t a = batch_pipeline_bucketed_table_bytes(inst), b = batch_pipeline_rows_table_bytes(inst);
    return a > b ? a : b;
}

static size_t batch_pipeline_rows_table_bytes(const std::vector<BatchInst>& inst) {
    size_t ci = 0, ri = 0;
    for (const BatchInst& I : inst) {
        ci += (size_t)((I.nnz + kEntryTile - 1) / kEntryTile);
        ri += (size_t)((I.nrows + kRowTile - 1) / kRowTile);
    }
    return ((inst.size() * sizeof(BatchInst) + 255) & ~(size_t)255) + ((ci * sizeof(WorkItem) + 255) & ~(size_t)255) +
           ((ri * sizeof(WorkItem) + 255) & ~(size_t)255);
}

}  // namespace hyd

using namespace hyd;

// ------------------------------------------------------------------ C ABI
extern "C" int hyd_cuda_coo_sum_duplicates_i64(const int64_t* rows, const int64_t* cols, const int64_t* vals,
                                               int64_t nnz, int64_t* out_rows, int64_t* out_cols, int64_t* out_vals,
                                               int64_t* out_nnz, void* stream) {
    HYD_CHECK_ARG(nnz >= 0, "coo_sum_duplicates: negative nnz");
    HYD_CHECK_ARG(out_nnz != nullptr, "coo_sum_duplicates: null out_nnz");
    HYD_CHECK_ARG(nnz == 0 || (rows && cols && vals && out_rows && out_cols && out_vals),
                  "coo_sum_duplicates: null buffer");
    cudaStream_t s = as_stream(stream);
    if (nnz == 0) {
        HYD_CUDA_TRY(cudaMemsetAsync(out_nnz, 0, 8, s));
        return HYD_CUDA_OK;
    }
    Device* d = nullptr;
    HYD_TRY(device(&d));
    void* dev_flags = nullptr;
    HYD_TRY(device_buffer(d, "coo_flags", 2 * (size_t)nnz * 8, &dev_flags));
    long long* flags = static_cast<long long*>(dev_flags);
    long long* seg = flags + nnz;
    int64_t blocks = (nnz + 255) / 256;
    if (blocks > d->sm_count * 8) blocks = d->sm_count * 8;
    coo_head_flags_kernel<<<(unsigned)blocks, 256, 0, s>>>((const long long*)rows, (const long long*)cols, nnz, flags);
    HYD_TRY(launch_check("coo_head_flags"));
    HYD_TRY(scan_i64_launch(flags, seg, nnz, 0, false, true, s));
    HYD_CUDA_TRY(cudaMemsetAsync(out_rows, 0, (size_t)nnz * 8, s));
    HYD_CUDA_TRY(cudaMemsetAsync(out_cols, 0, (size_t)nnz * 8, s));
    HYD_CUDA_TRY(cudaMemsetAsync(out_vals, 0, (size_t)nnz * 8, s));
    coo_merge_kernel<<<(unsigned)blocks, 256, 0, s>>>((const long long*)rows, (const long long*)cols,
                                                      (const long long*)vals, nnz, seg, (long long*)out_rows,
                                                      (long long*)out_cols, (unsigned long long*)out_vals);
    HYD_TRY(launch_check("coo_merge"));
    HYD_CUDA_TRY(cudaMemcpyAsync(out_nnz, seg + nnz - 1, 8, cudaMemcpyDeviceToDevice, s));
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_csr_from_sorted_coo_i64(int64_t nrows, int64_t nnz, const int64_t* rows, const int64_t* cols,
                                                const int64_t* vals, int64_t* row_ptr, int64_t* col_idx,
                                                int64_t* out_vals, void* stream) {
    HYD_CHECK_ARG(nrows >= 0 && nnz >= 0, "csr_from_sorted_coo: negative size");
    HYD_CHECK_ARG(row_ptr != nullptr, "csr_from_sorted_coo: null row_ptr");
    HYD_CHECK_ARG(nnz == 0 || (rows && cols && vals && col_idx && out_vals), "csr_from_sorted_coo: null buffer");
    cudaStream_t s = as_stream(stream);
    Device* d = nullptr;
    HYD_TRY(device(&d));
    if (nrows == 0) {
        HYD_CUDA_TRY(cudaMemsetAsync(row_ptr, 0, 8, s));
        if (nnz > 0) {
            // every entry's row is out of range
            csr_count_kernel<<<1, 32, 0, s>>>((const long long*)rows, nnz, 0, nullptr, d->d_err);
            HYD_TRY(launch_check("csr_count"));
        }
        return HYD_CUDA_OK;
    }
    void* buf = nullptr;
    HYD_TRY(device_buffer(d, "csr_counts", (size_t)nrows * 8, &buf));
    unsigned long long* counts = static_cast<unsigned long long*>(buf);
    HYD_CUDA_TRY(cudaMemsetAsync(counts, 0, (size_t)nrows * 8, s));
    int64_t blocks = (nnz + 255) / 256;
    if (blocks > d->sm_count * 8) blocks = d->sm_count * 8;
    if (blocks < 1) blocks = 1;
    if (nnz > 0) {
        csr_count_kernel<<<(unsigned)blocks, 256, 0, s>>>((const long long*)rows, nnz, nrows, counts, d->d_err);
        HYD_TRY(launch_check("csr_count"));
        copy_kernel<long long><<<(unsigned)blocks, 256, 0, s>>>((const long long*)cols, (long long*)col_idx, nnz);
        copy_kernel<long long><<<(unsigned)blocks, 256, 0, s>>>((const long long*)vals, (long long*)out_vals, nnz);
    }
    HYD_TRY(scan_i64_launch((const long long*)counts, (long long*)row_ptr, nrows, 0, false, false, s));
    set_last_kernel<<<1, 32, 0, s>>>((long long*)row_ptr, nrows, (const long long*)counts, (const long long*)row_ptr);
    return launch_check("csr_from_sorted_coo");
}

extern "C" int hyd_cuda_spmv_csr_f64(int64_t nrows, int64_t ncols, const int64_t* row_ptr, const int64_t* col_idx,
                                     const double* vals, const double* x, double* y, int lanes_per_row, void* stream) {
    HYD_CHECK_ARG(nrows >= 0 && ncols >= 0, "spmv_csr: negative size");
    HYD_CHECK_ARG(nrows == 0 || (row_ptr && y), "spmv_csr: null buffer");
    HYD_CHECK_ARG(lanes_per_row == 0 || lanes_per_row == 1 || lanes_per_row == 2 || lanes_per_row == 4 ||
                      lanes_per_row == 8 || lanes_per_row == 16 || lanes_per_row == 32,
                  "spmv_csr: lanes_per_row must be 0 (auto) or a power of two up to 32");
    if (nrows == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    int g = lanes_per_row ? lanes_per_row : 8;
    return spmv_dispatch<long long>(g, nrows, (const long long*)row_ptr, (const long long*)col_idx, vals, x, ncols, y, d,
                                    as_stream(stream));
}

extern "C" int hyd_cuda_spmv_csr_i32_f64(int64_t nrows, int64_t ncols, const int64_t* row_ptr, const int32_t* col_idx,
                                         const double* vals, const double* x, double* y, int lanes_per_row,
                                         void* stream) {
    HYD_CHECK_ARG(nrows >= 0 && ncols >= 0, "spmv_csr_i32: negative size");
    HYD_CHECK_ARG(nrows == 0 || (row_ptr && y), "spmv_csr_i32: null buffer");
    HYD_CHECK_ARG(lanes_per_row >= 0 && lanes_per_row <= 32 && (lanes_per_row & (lanes_per_row - 1)) == 0,
                  "spmv_csr_i32: lanes_per_row must be 0 (auto) or a power of two up to 32");
    if (nrows == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    int g = lanes_per_row ? lanes_per_row : 8;
    return spmv_dispatch<int>(g, nrows, (const long long*)row_ptr, (const int*)col_idx, vals, x, ncols, y, d,
                              as_stream(stream));
}

// Batched COO -> CSR -> SpMV.  `desc` is a HOST array of ninst x 3 int64
// (nrows, ncols, nnz); instances are concatenated in the device arrays in that
// order: rows/cols/vals/csr_cols/csr_vals by entries, x by ncols, y by nrows,
// row_ptr by nrows + 1.  row_ptr of each instance starts at 0.
extern "C" int hyd_cuda_batched_coo_csr_spmv_f64(int64_t ninst, const int64_t* desc, const int32_t* rows,
                                                 const int32_t* cols, const double* vals, const double* x,
                                                 int64_t* row_ptr, int32_t* csr_cols, double* csr_vals, double* y,
                                                 void* stream) {
    HYD_CHECK_ARG(ninst >= 0 && ninst < (1LL << 24), "batched_coo_csr_spmv: bad instance count");
    HYD_CHECK_ARG(ninst == 0 || desc != nullptr, "batched_coo_csr_spmv: null descriptor table");
    if (ninst == 0) return HYD_CUDA_OK;
    std::vector<BatchInst> inst((size_t)ninst);
    long long entries = 0, rows_total = 0, xs = 0;
    for (int64_t i = 0; i < ninst; ++i) {
        const long long nr = desc[3 * i], nc = desc[3 * i + 1], nz = desc[3 * i + 2];
        HYD_CHECK_ARG(nr >= 1 && nc >= 1 && nz >= 0 && nr < (1LL << 31) && nc < (1LL << 31),
                      "batched_coo_csr_spmv: instance %lld has a bad shape", (long long)i);
        BatchInst& I = inst[i];
        I.nrows = nr;
        I.ncols = nc;
        I.nnz = nz;
        I.rows = rows + entries;
        I.cols = cols + entries;
        I.vals = vals + entries;
        I.x = x + xs;
        I.row_ptr = (long long*)row_ptr + rows_total + i;
        I.csr_cols = csr_cols + entries;
        I.csr_vals = csr_vals + entries;
        I.y = y + rows_total;
        entries += nz;
        rows_total += nr;
        xs += nc;
    }
    HYD_CHECK_ARG(entries == 0 || (rows && cols && vals && csr_cols && csr_vals), "batched_coo_csr_spmv: null entries");
    HYD_CHECK_ARG(x && y && row_ptr, "batched_coo_csr_spmv: null x / y / row_ptr");
    return batch_pipeline(inst, "batch_tables", as_stream(stream), nullptr, 0);
}
