// sparse_bucket.cu -- the batched COO -> CSR -> SpMV pipeline, bucketed form.
//
// Same contract as batch_pipeline in sparse.cu (per instance: CSR of the
// entries sorted by (row, col), y = A x), organised so that no stage walks
// rows one dependent memory chain at a time:
//  1. count   per (instance, 8192-entry tile): a shared-memory histogram of
//             64-row buckets (row >> 6), flushed with one global red per
//             non-empty bucket;
//  2. scan    exclusive scan of the ~4e5 bucket counts gives every bucket's
//             first slot (instances are contiguous, so bucket starts are also
//             each instance's entry offsets);
//  3. split   per tile again: each entry gets its rank inside (tile, bucket)
//             from a shared-memory atomic, each (tile, bucket) reserves its run
//             with one global atomic, and the entry is written to the bucket's
//             region as a 32-bit key (row_in_bucket << 24 | col) plus its value
//             (the tile's values are prefetched into shared memory with
//             cp.async while the ranks and reservations are computed);
//  4. bucket  one CTA per bucket: its entries (at most 2048 in the fast kernel)
//             are counting-sorted by row into shared memory (64 counters), then
//             each warp takes rows, sorts a row by column in registers (bitonic
//             network over shuffles), writes its CSR columns/values and computes
//             its SpMV; the row pointers are the shared row offsets.  Buckets
//             above 2048 entries (64 rows x at most 256) go to an overflow list
//             handled by a block-wide bitonic sort in 96 KB of shared memory.
// The work lists of the stages (one item per (instance, tile) and per
// (instance, bucket)) are written on the device; only the instance table
// crosses from the host.
// Requires ncols < 2^24 (24-bit column field) and at most 256 entries per row.
#include <climits>
#include <cstring>
#include <vector>

#include "batch.cuh"
#include "hyd_common.cuh"

namespace hyd {

int scan_i64_launch(const long long* in, long long* out, int64_t n, long long init, bool reverse,
                    bool inclusive, cudaStream_t stream);

constexpr int kBkThreads = 512;
constexpr int kBkShift = 6;                  // 64 rows per bucket
constexpr int kBkRows = 1 << kBkShift;
constexpr int kBkCap = kBkRows * 256;        // entries per bucket at most (256 per row)
constexpr int kTileEntries = 8192;           // entries per count/split work item
constexpr int kMaxSmemBuckets = 4096;        // per instance (2^18 rows)

struct BkInst {
    long long nrows, ncols, nnz;
    long long bucket_base;  // first bucket in the batch-wide bucket space
    long long nbuckets;
    long long tile_base;    // first entry tile in the batch-wide tile list
    long long scan_base;    // entries of all earlier instances
    const int* rows;
    const int* cols;
    const double* vals;
    const double* x;
    long long* row_ptr;
    int* csr_cols;
    double* csr_vals;
    double* y;
};

struct BkItem {
    int inst;
    int tile;  // entry tile (stages 1, 3) or bucket index (stage 4)
};

__device__ __forceinline__ bool bk_next(unsigned* cursor, unsigned nitems, unsigned& item) {
    __shared__ unsigned sh_item;
    if (threadIdx.x == 0) sh_item = atomicAdd(cursor, 1u);
    __syncthreads();
    item = sh_item;
    __syncthreads();
    return item < nitems;
}

// Stage 1.
__global__ void __launch_bounds__(kBkThreads) bk_count_kernel(const BkInst* __restrict__ inst,
                                                              const BkItem* __restrict__ items, unsigned nitems,
                                                              unsigned* cursor, unsigned* __restrict__ bcount,
                                                              unsigned* err) {
    __shared__ unsigned hist[kMaxSmemBuckets];
    unsigned it;
    bool bad = false;
    while (bk_next(cursor, nitems, it)) {
        const BkItem w = items[it];
        const BkInst I = inst[w.inst];
        const bool smem = I.nbuckets <= kMaxSmemBuckets;
        if (smem)
            for (int b = threadIdx.x; b < I.nbuckets; b += kBkThreads) hist[b] = 0u;
        __syncthreads();
        const long long t0 = (long long)w.tile * kTileEntries;
        const long long t1 = t0 + kTileEntries < I.nnz ? t0 + kTileEntries : I.nnz;
        // all of this thread's rows first (read-only loads, all in flight at
        // once), then the counting: a load next to an atomic would otherwise
        // wait for it, one memory round trip per entry
        int rr[kTileEntries / kBkThreads];
#pragma unroll
        for (int j = 0; j < kTileEntries / kBkThreads; ++j) {
            const long long k = t0 + threadIdx.x + (long long)j * kBkThreads;
            rr[j] = k < t1 ? __ldg(I.rows + k) : INT_MIN;
        }
#pragma unroll
        for (int j = 0; j < kTileEntries / kBkThreads; ++j) {
            const int r = rr[j];  // columns are checked by the split, which reads them anyway
            if (r == INT_MIN && t0 + threadIdx.x + (long long)j * kBkThreads >= t1) continue;
            if (r < 0 || r >= I.nrows) {
                bad = true;
                continue;
            }
            if (smem) atomicAdd(&hist[r >> kBkShift], 1u);
            else atomicAdd(&bcount[I.bucket_base + (r >> kBkShift)], 1u);
        }
        __syncthreads();
        if (smem)
            for (int b = threadIdx.x; b < I.nbuckets; b += kBkThreads)
                if (hist[b]) atomicAdd(&bcount[I.bucket_base + b], hist[b]);
        __syncthreads();
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// The work lists of the count/split stages (one item per (instance, entry
// tile)) and of the bucket stage (one per (instance, bucket)), written on the
// device: block i writes instance i's items at its tile_base / bucket_base.
__global__ void bk_items_kernel(const BkInst* __restrict__ inst, int64_t ninst, BkItem* __restrict__ tiles,
                                BkItem* __restrict__ buckets) {
    for (int64_t i = blockIdx.x; i < ninst; i += gridDim.x) {
        const BkInst I = inst[i];
        const long long nt = (I.nnz + kTileEntries - 1) / kTileEntries;
        for (long long t = threadIdx.x; t < nt; t += blockDim.x) tiles[I.tile_base + t] = BkItem{(int)i, (int)t};
        for (long long b = threadIdx.x; b < I.nbuckets; b += blockDim.x)
            buckets[I.bucket_base + b] = BkItem{(int)i, (int)b};
    }
}

__global__ void bk_widen_kernel(const unsigned* __restrict__ c, long long* __restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = c[i];
}

// Stage 3.
constexpr int kSplitPer = kTileEntries / kBkThreads;  // 16 entries per thread
// The tile's values are copied into shared memory with cp.async as soon as
// the tile starts (8 bytes per copy, each thread the slots it later reads), so
// no global load is left on the path from the reservations to the stores.
constexpr size_t kSplitSmem = (size_t)kTileEntries * 8;  // 64 KB of values

__device__ __forceinline__ void cp_async_8(void* smem_dst, const void* gsrc) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(smem_dst)),
                 "l"(gsrc)
                 : "memory");
}

__global__ void __launch_bounds__(kBkThreads, 2) bk_split_kernel(const BkInst* __restrict__ inst,
                                                              const BkItem* __restrict__ items, unsigned nitems,
                                                              unsigned* cursor, const long long* __restrict__ bstart,
                                                              unsigned* __restrict__ bfill,
                                                              uint4* __restrict__ rec_out, unsigned* err) {
    __shared__ unsigned hist[kMaxSmemBuckets];
    __shared__ unsigned gbase[kMaxSmemBuckets];  // batch-wide slots (< 2^32, checked on the host)
    extern __shared__ __align__(16) double split_vals[];
    unsigned it;
    bool bad = false;
    while (bk_next(cursor, nitems, it)) {
        const BkItem w = items[it];
        const BkInst I = inst[w.inst];
        const bool smem = I.nbuckets <= kMaxSmemBuckets;
        const long long t0 = (long long)w.tile * kTileEntries;
        const long long t1 = t0 + kTileEntries < I.nnz ? t0 + kTileEntries : I.nnz;
#pragma unroll
        for (int j = 0; j < kSplitPer; ++j) {
            const int q = threadIdx.x + j * kBkThreads;
            if (t0 + q < t1) cp_async_8(split_vals + q, I.vals + t0 + q);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        if (smem)
            for (int b = threadIdx.x; b < I.nbuckets; b += kBkThreads) hist[b] = 0u;
        __syncthreads();
        unsigned key[kSplitPer], rank[kSplitPer];
        int bucket[kSplitPer];
        // the rows and columns of all this thread's entries first (read-only
        // loads, all in flight at once), then the ranking atomics
#pragma unroll
        for (int j = 0; j < kSplitPer; ++j) {
            const long long k = t0 + threadIdx.x + (long long)j * kBkThreads;
            bucket[j] = k < t1 ? __ldg(I.rows + k) : -1;
            key[j] = k < t1 ? (unsigned)__ldg(I.cols + k) : 0u;
        }
#pragma unroll
        for (int j = 0; j < kSplitPer; ++j) {
            const long long k = t0 + threadIdx.x + (long long)j * kBkThreads;
            const int r = bucket[j], c = (int)key[j];
            bucket[j] = -1;
            if (k < t1) {
                if (c < 0 || c >= I.ncols) bad = true;                 // (rows were checked by the count)
                if (r >= 0 && r < I.nrows && c >= 0 && c < I.ncols) {
                    bucket[j] = r >> kBkShift;
                    key[j] = ((unsigned)(r & (kBkRows - 1)) << 24) | (unsigned)c;
                    if (smem) rank[j] = atomicAdd(&hist[bucket[j]], 1u);
                }
            }
        }
        __syncthreads();
        if (smem) {
            // reserve this tile's run in every non-empty bucket; the atomics of
            // one thread are independent, so they are all issued before any
            // result is used (one memory round trip instead of eight)
            constexpr int kPerThread = kMaxSmemBuckets / kBkThreads;
            unsigned got[kPerThread];
#pragma unroll
            for (int q = 0; q < kPerThread; ++q) {
                const int b = threadIdx.x + q * kBkThreads;
                const unsigned c = b < I.nbuckets ? hist[b] : 0u;
                got[q] = c ? atomicAdd(&bfill[I.bucket_base + b], c) : 0u;
            }
#pragma unroll
            for (int q = 0; q < kPerThread; ++q) {
                const int b = threadIdx.x + q * kBkThreads;
                if (b < I.nbuckets && hist[b]) gbase[b] = (unsigned)(bstart[I.bucket_base + b] + got[q]);
            }
        }
        __syncthreads();
        // this thread's values have landed in shared memory (its own copies)
        asm volatile("cp.async.wait_all;" ::: "memory");
#pragma unroll
        for (int j = 0; j < kSplitPer; ++j) {
            if (bucket[j] < 0) continue;
            const int q = threadIdx.x + j * kBkThreads;
            const long long k = t0 + q;
            const double v = split_vals[q];
            const long long pos = smem ? (long long)gbase[bucket[j]] + rank[j]
                                       : bstart[I.bucket_base + bucket[j]] +
                                             atomicAdd(&bfill[I.bucket_base + bucket[j]], 1u);
            // one 16-byte record: the key, the entry's COO position (orders
            // equal (row, col) keys) and the value
            rec_out[pos] = make_uint4(key[j], (unsigned)k, (unsigned)__double2loint(v), (unsigned)__double2hiint(v));
        }
        __syncthreads();
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// ---- stage 4 ------------------------------------------------------------------
constexpr int kBkSmallThreads = 256;
constexpr int kBkSmallWarps = kBkSmallThreads / 32;
constexpr int kBkSmallCap = 2048;  // entries of a bucket handled in the fast kernel
constexpr int kBkRounds = kBkSmallCap / kBkSmallThreads;  // 32-element rounds per warp
// two (key, index) buffers, per-(warp, digit) counts, digit bases
constexpr size_t kBkSmallSmem = (size_t)kBkSmallCap * 12 + (size_t)kBkSmallWarps * 256 * 4 + 256 * 4;

// With invalid entries in a batch (reported by the count and split stages) a
// bucket's count can include an entry whose record the split did not write
// (a valid row with an invalid column): every column is bounded by ncols
// before x is read, so such a slot cannot index outside x.
//
// Equal (row, col) keys must keep their COO order (the runtime's stable
// sort_indices).  The split's order inside a bucket is arbitrary, so after the
// sort every run of equal keys is put in COO-position order (insertion sort
// by the thread that owns the run's first slot; duplicates are rare).
__device__ __forceinline__ double bk_rec_val(const uint4& r) { return __hiloint2double((int)r.w, (int)r.z); }

template <class IdxT>
__device__ __forceinline__ void bk_order_equal_keys(const unsigned* key, IdxT* pos, int E,
                                                    const uint4* __restrict__ rec) {
    for (int p = threadIdx.x; p + 1 < E; p += blockDim.x) {
        if (key[p + 1] != key[p] || (p > 0 && key[p - 1] == key[p])) continue;
        int q = p + 2;
        while (q < E && key[q] == key[p]) ++q;
        for (int i = p + 1; i < q; ++i) {
            const IdxT v = pos[i];
            const unsigned kv = rec[v].y;  // COO position
            int j = i - 1;
            while (j >= p && rec[pos[j]].y > kv) {
                pos[j + 1] = pos[j];
                --j;
            }
            pos[j + 1] = v;
        }
    }
}

// Fast path: a stable LSD radix sort of the bucket's keys (row_in_bucket <<
// cbits | col, 6 + cbits bits, 8 per pass) in shared memory; each warp owns
// consecutive positions, ranked in rounds of 32 with __match_any_sync so equal
// digits keep their order.  Row starts come from the row changes of the sorted
// keys.  Then CSR columns/values are written in sorted
// order (values gathered by index), and each warp computes the SpMV of its
// rows with lane i summing sorted positions i, i+32, ... (the same order as the
// other kernels).  Buckets above kBkSmallCap go to `overflow`.
constexpr int kBkSmallPerSm = 6;  // resident CTAs per SM
__global__ void __launch_bounds__(kBkSmallThreads, kBkSmallPerSm) bk_bucket_small_kernel(
    const BkInst* __restrict__ inst, const BkItem* __restrict__ items, unsigned nitems, unsigned* cursor,
    const long long* __restrict__ bstart, const unsigned* __restrict__ bcount, const uint4* __restrict__ rec_in,
    BkItem* __restrict__ overflow, unsigned* overflow_count, unsigned* err) {
    extern __shared__ __align__(16) unsigned char bks_smem[];
    unsigned* kbuf0 = reinterpret_cast<unsigned*>(bks_smem);
    unsigned* kbuf1 = kbuf0 + kBkSmallCap;
    unsigned short* ibuf0 = reinterpret_cast<unsigned short*>(kbuf1 + kBkSmallCap);
    unsigned short* ibuf1 = ibuf0 + kBkSmallCap;
    unsigned* wcount = reinterpret_cast<unsigned*>(ibuf1 + kBkSmallCap);  // [warps][256]
    unsigned* dbase = wcount + kBkSmallWarps * 256;                        // [256]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    unsigned it;
    bool bad = false;
    while (bk_next(cursor, nitems, it)) {
        const BkItem w = items[it];
        const BkInst I = inst[w.inst];
        const long long gb = I.bucket_base + w.tile;
        const int E = (int)bcount[gb];
        if (E > kBkSmallCap) {
            if (threadIdx.x == 0) overflow[atomicAdd(overflow_count, 1u)] = w;
            continue;  // uniform
        }
        const long long s0 = bstart[gb];
        const long long e0 = s0 - I.scan_base;
        const long long r0 = (long long)w.tile << kBkShift;
        const int nr = (int)((I.nrows - r0) < kBkRows ? (I.nrows - r0) : kBkRows);
        int cbits = 0;
        while ((1LL << cbits) < I.ncols) ++cbits;
        // key = row_in_bucket << cbits | col: 6 + cbits bits, 8 per pass
        const int passes = (kBkShift + cbits + 7) / 8;
        for (int i = threadIdx.x; i < E; i += kBkSmallThreads) {
            const unsigned k = rec_in[s0 + i].x;
            kbuf0[i] = ((k >> 24) << cbits) | (k & 0xFFFFFFu);
            ibuf0[i] = (unsigned short)i;
        }
        // positions split evenly over the warps (whole 32-element rounds); warp
        // order is position order, so ranks stay stable
        const int chunk = (((E + kBkSmallWarps - 1) / kBkSmallWarps) + 31) & ~31;
        const int rounds = chunk / 32;
        unsigned* kin = kbuf0;
        unsigned* kout = kbuf1;
        unsigned short* iin = ibuf0;
        unsigned short* iout = ibuf1;
        __syncthreads();
        for (int pass = 0; pass < passes; ++pass) {
            const int shift = 8 * pass;
            for (int i = threadIdx.x; i < kBkSmallWarps * 256; i += kBkSmallThreads) wcount[i] = 0u;
            __syncthreads();
            unsigned rk[kBkRounds];
            unsigned dg[kBkRounds];
#pragma unroll
            for (int r = 0; r < kBkRounds; ++r) {
                if (r >= rounds) break;  // warp-uniform
                const int pos = warp * chunk + r * 32 + lane;
                const bool ok = pos < E && pos < (warp + 1) * chunk;
                const unsigned d = ok ? ((kin[pos] >> shift) & 0xFFu) : 0x100u;
                dg[r] = d;
                const unsigned peers = __match_any_sync(0xffffffffu, d);
                unsigned prior = 0;
                if (ok) prior = wcount[warp * 256 + d];
                __syncwarp();
                rk[r] = prior + __popc(peers & lt);
                if (ok && (peers & lt) == 0u) wcount[warp * 256 + d] = prior + __popc(peers);
                __syncwarp();
            }
            __syncthreads();
            // digit totals, their exclusive scan, then per-(warp, digit) bases
            const int dgt = threadIdx.x;  // 256 threads <-> 256 digits
            unsigned tot = 0;
#pragma unroll
            for (int ww = 0; ww < kBkSmallWarps; ++ww) tot += wcount[ww * 256 + dgt];
            unsigned incl = tot;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += y;
            }
            if (lane == 31) dbase[warp] = incl;
            __syncthreads();
            unsigned wpre = 0;
            for (int ww = 0; ww < warp; ++ww) wpre += dbase[ww];
            __syncthreads();
            unsigned run = wpre + incl - tot;  // exclusive base of digit dgt
            dbase[dgt] = run;
#pragma unroll
            for (int ww = 0; ww < kBkSmallWarps; ++ww) {
                const unsigned c = wcount[ww * 256 + dgt];
                wcount[ww * 256 + dgt] = run;
                run += c;
            }
            __syncthreads();
#pragma unroll
            for (int r = 0; r < kBkRounds; ++r) {
                if (r >= rounds) break;
                const int pos = warp * chunk + r * 32 + lane;
                if (pos < E && pos < (warp + 1) * chunk) {
                    const unsigned dst = wcount[warp * 256 + dg[r]] + rk[r];
                    kout[dst] = kin[pos];
                    iout[dst] = iin[pos];
                }
            }
            __syncthreads();
            unsigned* tk = kin; kin = kout; kout = tk;
            unsigned short* ti = iin; iin = iout; iout = ti;
        }
        // kin/iin: sorted by (row, col); row starts from the row changes
        const unsigned cmask = (1u << cbits) - 1u;
        for (int p = threadIdx.x; p <= E; p += kBkSmallThreads) {
            const int rp = p == 0 ? -1 : (int)(kin[p - 1] >> cbits);
            const int rc = p == E ? kBkRows : (int)(kin[p] >> cbits);
            for (int r = rp + 1; r <= rc && r < kBkRows; ++r) dbase[r] = (unsigned)p;
        }
        bk_order_equal_keys(kin, iin, E, rec_in + s0);
        __syncthreads();
        for (int p = threadIdx.x; p < E; p += kBkSmallThreads) {
            I.csr_cols[e0 + p] = (int)(kin[p] & cmask);
            I.csr_vals[e0 + p] = bk_rec_val(rec_in[s0 + iin[p]]);
        }
        for (int r = threadIdx.x; r <= nr; r += kBkSmallThreads) {
            if (r < nr) I.row_ptr[r0 + r] = e0 + dbase[r];
            else if (r0 + nr == I.nrows) I.row_ptr[I.nrows] = I.nnz;
        }
        // SpMV.  Rows of at most 32 entries: one lane per row, summed in column
        // order (warps 0-1 cover the bucket's 64 rows).  Longer rows: a warp,
        // lane i summing positions i, i+32, ..., then a fixed xor tree.  (On
        // GB300 every FP64 warp instruction holds the FP64 pipe for ~64 cycles,
        // so a tree per short row would cost more than the row itself.)
        auto row_end = [&](int r) { return r + 1 < nr ? (int)dbase[r + 1] : E; };
        if (warp < kBkRows / 32) {
            const int r = warp * 32 + lane;
            if (r < nr) {
                const int a = (int)dbase[r], bb = row_end(r);
                if (bb - a <= 32) {
                    double acc = 0.0;
                    for (int p = a; p < bb; ++p) {
                        const unsigned c = kin[p] & cmask;
                        acc = fma(bk_rec_val(rec_in[s0 + iin[p]]), c < I.ncols ? I.x[c] : 0.0, acc);
                    }
                    I.y[r0 + r] = acc;
                }
            }
        }
        for (int r = warp; r < nr; r += kBkSmallWarps) {
            const int a = (int)dbase[r], bb = row_end(r);
            if (bb - a <= 32) continue;  // warp-uniform
            if (bb - a > 256) bad = true;  // a row above 256 entries: outside the contract
            double acc = 0.0;
            for (int p = a + lane; p < bb; p += 32) {
                const unsigned c = kin[p] & cmask;
                acc = fma(bk_rec_val(rec_in[s0 + iin[p]]), c < I.ncols ? I.x[c] : 0.0, acc);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) I.y[r0 + r] = acc;
        }
        __syncthreads();
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// Large buckets (up to 64 rows x 256): one CTA sorts the bucket's keys with a
// block-wide bitonic network in shared memory.  Reads its item count from
// device memory (filled by the fast kernel).
constexpr size_t kBkSmem = (size_t)kBkCap * 6 + 1024;

__global__ void __launch_bounds__(kBkThreads) bk_bucket_kernel(const BkInst* __restrict__ inst,
                                                               const BkItem* __restrict__ items,
                                                               const unsigned* nitems_dev, unsigned* cursor,
                                                               const long long* __restrict__ bstart,
                                                               const unsigned* __restrict__ bcount,
                                                               const uint4* __restrict__ rec_in, unsigned* err) {
    extern __shared__ __align__(16) unsigned char bk_smem[];
    unsigned* key = reinterpret_cast<unsigned*>(bk_smem);
    unsigned short* idx = reinterpret_cast<unsigned short*>(bk_smem + (size_t)kBkCap * 4);
    __shared__ int rstart[kBkRows + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned nitems = *nitems_dev;
    unsigned it;
    bool bad = false;
    while (bk_next(cursor, nitems, it)) {
        const BkItem w = items[it];
        const BkInst I = inst[w.inst];
        const long long gb = I.bucket_base + w.tile;
        const int E = (int)bcount[gb];
        const long long s0 = bstart[gb];        // batch-wide slot of the bucket's first entry
        const long long e0 = s0 - I.scan_base;  // instance-relative
        const long long r0 = (long long)w.tile << kBkShift;
        const int nr = (int)((I.nrows - r0) < kBkRows ? (I.nrows - r0) : kBkRows);
        if (E > kBkCap) {  // a row above 256 entries: outside the contract
            bad = true;
            continue;
        }
        int P = 1;
        while (P < E) P <<= 1;
        for (int i = threadIdx.x; i < P; i += kBkThreads) {
            key[i] = i < E ? rec_in[s0 + i].x : 0xFFFFFFFFu;
            idx[i] = (unsigned short)i;
        }
        __syncthreads();
        for (int size = 2; size <= P; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = threadIdx.x; i < P / 2; i += kBkThreads) {
                    const int lo = 2 * i - (i & (stride - 1));
                    const int hi = lo + stride;
                    const bool up = (lo & size) == 0;
                    const unsigned a = key[lo], b = key[hi];
                    if ((a > b) == up) {
                        key[lo] = b;
                        key[hi] = a;
                        const unsigned short t = idx[lo];
                        idx[lo] = idx[hi];
                        idx[hi] = t;
                    }
                }
                __syncthreads();
            }
        }
        for (int p = threadIdx.x; p <= E; p += kBkThreads) {
            const int rp = p == 0 ? -1 : (int)(key[p - 1] >> 24);
            const int rc = p == E ? nr : (int)(key[p] >> 24);
            for (int r = rp + 1; r <= rc && r <= nr; ++r) rstart[r] = p;
        }
        bk_order_equal_keys(key, idx, E, rec_in + s0);  // the bitonic network is not stable
        __syncthreads();
        for (int p = threadIdx.x; p < E; p += kBkThreads) {
            I.csr_cols[e0 + p] = (int)(key[p] & 0xFFFFFFu);
            I.csr_vals[e0 + p] = bk_rec_val(rec_in[s0 + idx[p]]);
        }
        for (int r = threadIdx.x; r <= nr; r += kBkThreads) {
            if (r < nr) I.row_ptr[r0 + r] = e0 + rstart[r];
            else if (r0 + nr == I.nrows) I.row_ptr[I.nrows] = I.nnz;
        }
        // SpMV as in the fast kernel: short rows one lane each, long rows a warp
        if (warp < kBkRows / 32) {
            const int r = warp * 32 + lane;
            if (r < nr && rstart[r + 1] - rstart[r] <= 32) {
                double acc = 0.0;
                for (int p = rstart[r]; p < rstart[r + 1]; ++p) {
                    const unsigned c = key[p] & 0xFFFFFFu;
                    acc = fma(bk_rec_val(rec_in[s0 + idx[p]]), c < I.ncols ? I.x[c] : 0.0, acc);
                }
                I.y[r0 + r] = acc;
            }
        }
        for (int r = warp; r < nr; r += kBkThreads / 32) {
            if (rstart[r + 1] - rstart[r] <= 32) continue;  // warp-uniform
            double acc = 0.0;
            for (int p = rstart[r] + lane; p < rstart[r + 1]; p += 32) {
                const unsigned c = key[p] & 0xFFFFFFu;
                acc = fma(bk_rec_val(rec_in[s0 + idx[p]]), c < I.ncols ? I.x[c] : 0.0, acc);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) I.y[r0 + r] = acc;
        }
        __syncthreads();
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// Bucketed pipeline; returns HYD_CUDA_ERR_UNSUPPORTED (nothing launched) when a
// batch falls outside its limits so the caller can take the row-atomic path.
int batch_pipeline_bucketed(std::vector<BatchInst>& bi, const char* key, cudaStream_t s, void* staging,
                            size_t staging_bytes) {
    Device* d = nullptr;
    HYD_TRY(device(&d));
    std::vector<BkInst> inst(bi.size());
    long long nb_total = 0, entries = 0, nt_total = 0;
    for (size_t i = 0; i < bi.size(); ++i) {
        const BatchInst& B = bi[i];
        if (B.ncols >= (1LL << 24) || B.nrows >= (1LL << 31)) return HYD_CUDA_ERR_UNSUPPORTED;
        BkInst& I = inst[i];
        I.nrows = B.nrows;
        I.ncols = B.ncols;
        I.nnz = B.nnz;
        I.nbuckets = (B.nrows + kBkRows - 1) / kBkRows;
        I.bucket_base = nb_total;
        I.scan_base = entries;
        I.rows = B.rows;
        I.cols = B.cols;
        I.vals = B.vals;
        I.x = B.x;
        I.row_ptr = B.row_ptr;
        I.csr_cols = B.csr_cols;
        I.csr_vals = B.csr_vals;
        I.y = B.y;
        I.tile_base = nt_total;
        nt_total += (B.nnz + kTileEntries - 1) / kTileEntries;
        nb_total += I.nbuckets;
        entries += B.nnz;
    }
    if (nb_total >= (1LL << 31) || nt_total >= (1LL << 31) || entries >= (1LL << 32))
        return HYD_CUDA_ERR_UNSUPPORTED;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t inst_b = al(inst.size() * sizeof(BkInst)), tiles_b = al((size_t)nt_total * sizeof(BkItem)),
                 bk_b = al((size_t)nb_total * sizeof(BkItem));
    const size_t cnt_b = al((size_t)nb_total * 4), wide_b = al((size_t)nb_total * 8);
    const size_t vals_b = al((size_t)entries * 8);
    void* buf = nullptr;
    HYD_TRY(device_buffer(d, key, inst_b + tiles_b + 2 * bk_b + 2 * cnt_b + 2 * wide_b + vals_b + vals_b + 256,
                          &buf));
    unsigned char* b = static_cast<unsigned char*>(buf);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = b + off;
        off += bytes;
        return p;
    };
    BkInst* d_inst = reinterpret_cast<BkInst*>(take(inst_b));
    BkItem* d_tiles = reinterpret_cast<BkItem*>(take(tiles_b));
    BkItem* d_bk = reinterpret_cast<BkItem*>(take(bk_b));
    unsigned* bcount = reinterpret_cast<unsigned*>(take(cnt_b));
    unsigned* bfill = reinterpret_cast<unsigned*>(take(cnt_b));
    long long* wide = reinterpret_cast<long long*>(take(wide_b));
    long long* bstart = reinterpret_cast<long long*>(take(wide_b));
    uint4* recs = reinterpret_cast<uint4*>(take(2 * vals_b));  // (key, COO position, value) per entry
    BkItem* overflow = reinterpret_cast<BkItem*>(take(bk_b));
    unsigned* cursors = reinterpret_cast<unsigned*>(take(256));
    // only the instance table crosses from the host; the work lists are
    // written by bk_items_kernel
    const bool async_tables = staging != nullptr && staging_bytes >= inst_b;
    if (async_tables) {
        memcpy(staging, inst.data(), inst.size() * sizeof(BkInst));
        HYD_CUDA_TRY(cudaMemcpyAsync(d_inst, staging, inst.size() * sizeof(BkInst), cudaMemcpyHostToDevice, s));
    } else {
        HYD_CUDA_TRY(cudaMemcpyAsync(d_inst, inst.data(), inst.size() * sizeof(BkInst), cudaMemcpyHostToDevice, s));
    }
    {
        const int64_t ni = (int64_t)inst.size();
        const unsigned g = (unsigned)(ni < 4096 ? ni : 4096);
        bk_items_kernel<<<g, 256, 0, s>>>(d_inst, ni, d_tiles, d_bk);
        HYD_TRY(launch_check("bk_items"));
    }
    const size_t n_tiles = (size_t)nt_total, n_buckets = (size_t)nb_total;
    HYD_CUDA_TRY(cudaMemsetAsync(bcount, 0, 2 * cnt_b, s));  // bcount and bfill
    HYD_CUDA_TRY(cudaMemsetAsync(cursors, 0, 64, s));
    const unsigned grid = (unsigned)(d->sm_count * 2);
    if (n_tiles) {
        bk_count_kernel<<<grid, kBkThreads, 0, s>>>(d_inst, d_tiles, (unsigned)n_tiles, cursors + 0, bcount,
                                                    d->d_err);
        HYD_TRY(launch_check("bk_count"));
    }
    bk_widen_kernel<<<grid, 256, 0, s>>>(bcount, wide, nb_total);
    HYD_TRY(launch_check("bk_widen"));
    HYD_TRY(scan_i64_launch(wide, bstart, nb_total, 0, false, false, s));
    if (n_tiles) {
        HYD_TRY(configure_kernel((const void*)bk_split_kernel, d, false));
        bk_split_kernel<<<grid, kBkThreads, kSplitSmem, s>>>(d_inst, d_tiles, (unsigned)n_tiles, cursors + 1, bstart,
                                                             bfill, recs, d->d_err);
        HYD_TRY(launch_check("bk_split"));
    }
    HYD_TRY(configure_kernel((const void*)bk_bucket_small_kernel, d, false));
    bk_bucket_small_kernel<<<(unsigned)(d->sm_count * kBkSmallPerSm), kBkSmallThreads, kBkSmallSmem, s>>>(
        d_inst, d_bk, (unsigned)n_buckets, cursors + 2, bstart, bcount, recs, overflow, cursors + 4, d->d_err);
    HYD_TRY(launch_check("bk_bucket_small"));
    HYD_TRY(configure_kernel((const void*)bk_bucket_kernel, d, false));
    bk_bucket_kernel<<<grid, kBkThreads, kBkSmem, s>>>(d_inst, overflow, cursors + 4, cursors + 3, bstart, bcount,
                                                       recs, d->d_err);
    HYD_TRY(launch_check("bk_bucket_large"));
    if (!async_tables) HYD_CUDA_TRY(cudaStreamSynchronize(s));
    return HYD_CUDA_OK;
}

size_t batch_pipeline_bucketed_table_bytes(const std::vector<BatchInst>& bi) {
    return (bi.size() * sizeof(BkInst) + 255) & ~(size_t)255;
}

}  // namespace hyd
