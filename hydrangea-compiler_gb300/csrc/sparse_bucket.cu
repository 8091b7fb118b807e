// sparse_bucket.cu -- the batched COO -> CSR -> SpMV pipeline, bucketed form.
//
// Same contract as batch_pipeline in sparse.cu (per instance: CSR of the
// entries sorted by (row, col), y = A x), organised so that no stage walks
// rows one dependent memory chain at a time:
//  1. count   per CTA, a contiguous range of (instance, 8192-entry tile)
//             items: a shared-memory histogram of 64-row buckets (row >> 6),
//             flushed with one global red per non-empty bucket when the
//             instance changes;
//  2. scan    exclusive scan of the ~4e5 bucket counts gives every bucket's
//             first slot (instances are contiguous, so bucket starts are also
//             each instance's entry offsets);
//  3. split   per tile again: each entry gets its rank inside (tile, bucket)
//             from a shared-memory atomic, each (tile, bucket) reserves its run
//             with one global atomic, and the entry is written to the bucket's
//             region as a 32-bit key (row_in_bucket << 24 | col) plus its value
//             (the tile's values are prefetched into shared memory with
//             cp.async while the ranks and reservations are computed);
//  4. bucket  one warp per bucket (at most 2048 entries, ncols <= 2^18): a
//             stable LSD radix sort of the packed (row, col) keys in shared
//             memory, the CSR columns/values written in sorted order and the
//             row pointers from the row changes.  Larger buckets go to an
//             overflow list sorted by a block-wide bitonic network;
//  5. spmv    one warp per 256-row chunk of an instance: the rows are ordered
//             by length in shared memory and each lane sums one row's fma
//             chain in column order, 32 rows of similar length at a time.
// The work lists of the stages (one item per (instance, tile), per (instance,
// bucket) and per (instance, 256-row chunk)) are written on the device; only
// the instance table crosses from the host.
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
    long long chunk_base;   // first 256-row SpMV chunk in the batch-wide chunk list
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

// Stage 1.  Each CTA counts a contiguous range of the tile list (the tiles of
// an instance are consecutive there), keeping its shared-memory bucket counts
// across the tiles of one instance and flushing them with one global red per
// non-empty bucket when the instance changes.  A flush per tile issued about
// one red per two entries for the largest instances, and the L2 atomics bound
// the kernel.  The counts are zero whenever they are not in use (the flush
// zeroes what it reads).
constexpr int kCountPerSm = 4;
__global__ void __launch_bounds__(kBkThreads, kCountPerSm) bk_count_kernel(const BkInst* __restrict__ inst,
                                                              const BkItem* __restrict__ items, unsigned nitems,
                                                              unsigned* __restrict__ bcount, unsigned* err) {
    __shared__ unsigned hist[kMaxSmemBuckets];
    for (int b = threadIdx.x; b < kMaxSmemBuckets; b += kBkThreads) hist[b] = 0u;
    const unsigned per = (nitems + gridDim.x - 1) / gridDim.x;
    const unsigned i0 = blockIdx.x * per;
    const unsigned i1 = i0 + per < nitems ? i0 + per : nitems;
    int cur = -1;
    long long cur_base = 0;
    int cur_nb = 0;
    bool bad = false;
    auto flush = [&]() {
        if (cur >= 0 && cur_nb <= kMaxSmemBuckets)
            for (int b = threadIdx.x; b < cur_nb; b += kBkThreads) {
                const unsigned c = hist[b];
                if (c) {
                    atomicAdd(&bcount[cur_base + b], c);
                    hist[b] = 0u;
                }
            }
    };
    __syncthreads();
    for (unsigned it = i0; it < i1; ++it) {
        const BkItem w = items[it];
        const BkInst I = inst[w.inst];
        if (w.inst != cur) {
            __syncthreads();  // the counting of the previous tile is complete
            flush();
            cur = w.inst;
            cur_base = I.bucket_base;
            cur_nb = (int)I.nbuckets;
            __syncthreads();  // the flush has read and zeroed every count
        }
        const bool smem = cur_nb <= kMaxSmemBuckets;
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
    }
    __syncthreads();
    flush();
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

constexpr int kSpRows = 256;  // rows per SpMV chunk

// The work lists of the count/split stages (one item per (instance, entry
// tile)), of the bucket stage (one per (instance, bucket)) and of the SpMV
// (one per (instance, 256-row chunk)), written on the device: block i writes
// instance i's items at its tile_base / bucket_base / chunk_base.
__global__ void bk_items_kernel(const BkInst* __restrict__ inst, int64_t ninst, BkItem* __restrict__ tiles,
                                BkItem* __restrict__ buckets, BkItem* __restrict__ chunks) {
    for (int64_t i = blockIdx.x; i < ninst; i += gridDim.x) {
        const BkInst I = inst[i];
        const long long nt = (I.nnz + kTileEntries - 1) / kTileEntries;
        const long long nc = (I.nrows + kSpRows - 1) / kSpRows;
        for (long long t = threadIdx.x; t < nt; t += blockDim.x) tiles[I.tile_base + t] = BkItem{(int)i, (int)t};
        for (long long b = threadIdx.x; b < I.nbuckets; b += blockDim.x)
            buckets[I.bucket_base + b] = BkItem{(int)i, (int)b};
        for (long long c = threadIdx.x; c < nc; c += blockDim.x) chunks[I.chunk_base + c] = BkItem{(int)i, (int)c};
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

// One warp per bucket: a warp sorts its own bucket with no block barrier, so
// fifteen independent buckets are in flight per SM.  (A CTA per ~800-entry
// bucket pays its fixed work -- zeroing and scanning a counter set per warp,
// five block barriers per radix pass -- once per bucket.)
//  * key24 = row_in_bucket << cbits | col, kept to its 6 + cbits <= 24 bits,
//    sorted by stable LSD passes of 8 bits (at most three);
//  * the digit counts of every pass are taken in one sweep when the keys are
//    loaded (the multiset of digits does not change between passes), as
//    16-bit counts packed two to a word (digits d and d + 128);
//  * pass 0 reads key24 with the implicit index = position and writes
//    (key24 >> 8) << 11 | index; later passes move that word, whose bits
//    8k + 3 ... hold digit k, so one 32-bit word per entry carries both the
//    remaining key and the entry index;
//  * each pass ranks 32 positions per round among the lanes holding the same
//    digit (bk_rank_pass), so equal digits keep their order;
//  * after the sort every slot's record is gathered once for its full key,
//    CSR column and value, 32 consecutive slots per step, which also gives
//    the row starts and any equal neighbouring keys; runs of equal keys are
//    then put in COO order.
// Row starts come from the masked keys, which are sorted on every bit they
// have whatever the records hold, so every row range stays inside [0, E].
// The pipeline runs it with room for 1536 entries per warp (fifteen warps per
// SM; 0.5% of the workload's buckets are larger).  Buckets above kCap, or of
// instances with more than 2^18
// columns, go to `overflow` (the block-wide kernel below).
constexpr int kBkWarpIdxBits = 11;   // entry index bits: buckets of at most 2048 entries
constexpr unsigned kBkWarpIdxMask = (1u << kBkWarpIdxBits) - 1u;
constexpr int kBkWarpMaxCbits = 24 - kBkShift;
constexpr int kBkWarpPerSm = 3;  // resident CTAs per SM
// per warp (32-bit words): two key buffers, packed digit counts of three
// passes, the running digit bases (later the row starts)
template <int kCap>
__host__ __device__ constexpr int bk_warp_words() { return 2 * kCap + 3 * 128 + 256; }
template <int kCap, int kWarps>
constexpr size_t bk_warp_smem() { return (size_t)kWarps * bk_warp_words<kCap>() * 4; }

// The sort key of a record: row_in_bucket << cbits | col, kept to its 6 + cbits
// bits (which change nothing for a valid entry, and keep every key's row
// below kBkRows whatever an unwritten slot holds).
__device__ __forceinline__ unsigned bk_key24(unsigned k, int cbits) {
    return (((k >> 24) << cbits) | (k & 0xFFFFFFu)) & ((1u << (kBkShift + cbits)) - 1u);
}

// One stable scatter pass of the warp sort: positions 0 .. E-1 of src, 32 per
// round, go to dst at base[digit] + (their rank among the round's lanes with
// the same digit); base[] holds the running digit offsets.  Lanes holding
// the same digit are found with one ballot per digit bit (the ALU pipe); a
// match instruction per round (the ADU pipe) kept that pipe 66% busy and was
// slower.  (Skipping the digit bits a pass cannot hold made no difference.)
__device__ __forceinline__ void bk_rank_pass(const unsigned* src, unsigned* dst, int E, int shift, bool first,
                                             unsigned* base, int lane, unsigned lt) {
    for (int p0 = 0; p0 < E; p0 += 32) {
        const int p = p0 + lane;
        const bool ok = p < E;
        const unsigned v = ok ? src[p] : 0u;
        const unsigned d = (v >> shift) & 0xFFu;
        unsigned peers = __ballot_sync(0xffffffffu, ok);
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            const unsigned bb = __ballot_sync(0xffffffffu, (d >> b) & 1u);
            peers &= ((d >> b) & 1u) ? bb : ~bb;
        }
        unsigned at = 0;
        if (ok) at = base[d];
        __syncwarp();
        if (ok) {
            const unsigned before = peers & lt;
            dst[at + __popc(before)] = first ? (((v >> 8) << kBkWarpIdxBits) | (unsigned)p) : v;
            if (before == 0u) base[d] = at + __popc(peers);
        }
        __syncwarp();
    }
}

template <int kCap, int kWarps>
__global__ void __launch_bounds__(kWarps * 32, kBkWarpPerSm) bk_bucket_warp_kernel(
    const BkInst* __restrict__ inst, const BkItem* __restrict__ items, unsigned nitems_host,
    const unsigned* nitems_dev, unsigned* cursor,
    const long long* __restrict__ bstart, const unsigned* __restrict__ bcount, const uint4* __restrict__ rec_in,
    BkItem* __restrict__ overflow, unsigned* overflow_count, unsigned* err) {
    extern __shared__ __align__(16) unsigned bkw_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    static_assert(kCap <= (1 << kBkWarpIdxBits), "entry indices must fit their field");
    unsigned* const a = bkw_smem + (size_t)warp * bk_warp_words<kCap>();
    unsigned* const b = a + kCap;
    unsigned* const hist = b + kCap;  // [3][128]
    // the item count: given, or read from device memory (a list another kernel filled)
    const unsigned nitems = nitems_dev ? *(volatile const unsigned*)nitems_dev : nitems_host;
    unsigned* const base = hist + 3 * 128;  // [256]; row starts [65] after the sort
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    for (;;) {
        unsigned it = 0;
        if (lane == 0) it = atomicAdd(cursor, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= nitems) break;
        const BkItem w = items[it];
        const BkInst I = inst[w.inst];
        const long long gb = I.bucket_base + w.tile;
        const int E = (int)bcount[gb];
        // bits of the largest column: the smallest c with 2^c >= ncols
        const int cbits = I.ncols > 1 ? 64 - __clzll((unsigned long long)(I.ncols - 1)) : 0;
        if (E > kCap || cbits > kBkWarpMaxCbits) {
            if (lane == 0) overflow[atomicAdd(overflow_count, 1u)] = w;
            continue;  // warp-uniform
        }
        const long long s0 = bstart[gb];
        const long long e0 = s0 - I.scan_base;
        const long long r0 = (long long)w.tile << kBkShift;
        const int nr = (int)((I.nrows - r0) < kBkRows ? (I.nrows - r0) : kBkRows);
        const int passes = (kBkShift + cbits + 7) >> 3;  // 1..3
        // keys and the digit counts of every pass
        // every lane's key words are in flight at once (4-byte cp.async of
        // each record's key field), so the bucket waits for one memory latency
        for (int p = lane; p < E; p += 32)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(a + p)),
                         "l"(&rec_in[s0 + p].x)
                         : "memory");
        asm volatile("cp.async.commit_group;" ::: "memory");
        for (int i = lane; i < 3 * 128; i += 32) hist[i] = 0u;
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncwarp();
        for (int p = lane; p < E; p += 32) {
            const unsigned key = bk_key24(a[p], cbits);
            a[p] = key;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (k < passes) {
                    const unsigned d = (key >> (8 * k)) & 0xFFu;
                    atomicAdd(&hist[k * 128 + (d & 127u)], (d & 128u) ? 0x10000u : 1u);
                }
            }
        }
        __syncwarp();
        unsigned* src = a;
        unsigned* dst = b;
        for (int k = 0; k < passes; ++k) {
            // exclusive scan of the 256 digit counts; lane l owns digits 8l .. 8l+7
            unsigned c[8], sum = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int d = 8 * lane + j;
                c[j] = (hist[k * 128 + (d & 127)] >> ((d & 128) ? 16 : 0)) & 0xFFFFu;
                sum += c[j];
            }
            unsigned incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            unsigned run = incl - sum;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                base[8 * lane + j] = run;
                run += c[j];
            }
            __syncwarp();
            const int shift = k == 0 ? 0 : 8 * k + 3;
            bk_rank_pass(src, dst, E, shift, k == 0, base, lane, lt);
            unsigned* t = src;
            src = dst;
            dst = t;
        }
        // src: entry indices in (row, col) order; dst: free for the keys
        unsigned* const ord = src;
        unsigned* const key = dst;
        const unsigned cmask = (1u << cbits) - 1u;
        // One pass over the sorted positions, 32 consecutive ones per warp step:
        // gather each record for its key, CSR column and value, and find the
        // row starts and any equal neighbouring keys from the neighbour's key
        // (a shuffle; the step before hands over its last key).
        unsigned* const rowb = base;  // [kBkRows + 1]
        constexpr int kG = 8;         // records in flight per lane
        unsigned prev_key = 0u;
        int prev_row = -1;  // row of the position before the current step (-1: none)
        bool dup = false;
        for (int c0 = 0; c0 < E; c0 += 32 * kG) {
            uint4 r[kG];
#pragma unroll
            for (int u = 0; u < kG; ++u) {
                const int p = c0 + 32 * u + lane;
                if (p < E) r[u] = rec_in[s0 + (ord[p] & kBkWarpIdxMask)];
            }
#pragma unroll
            for (int u = 0; u < kG; ++u) {
                const int p = c0 + 32 * u + lane;
                const bool in = p < E;
                unsigned k24 = 0u;
                if (in) {
                    k24 = bk_key24(r[u].x, cbits);
                    key[p] = k24;
                    I.csr_cols[e0 + p] = (int)(k24 & cmask);
                    I.csr_vals[e0 + p] = bk_rec_val(r[u]);
                }
                const int row = in ? (int)(k24 >> cbits) : kBkRows;
                const unsigned kup = __shfl_up_sync(0xffffffffu, k24, 1);
                const int rup = __shfl_up_sync(0xffffffffu, row, 1);
                const unsigned kprev = lane == 0 ? prev_key : kup;
                const int rprev = lane == 0 ? prev_row : rup;
                if (in) {
                    for (int rr = rprev + 1; rr <= row && rr < kBkRows; ++rr) rowb[rr] = (unsigned)p;
                    dup |= p > 0 && kprev == k24;
                }
                prev_key = __shfl_sync(0xffffffffu, k24, 31);
                prev_row = __shfl_sync(0xffffffffu, row, 31);
            }
        }
        __syncwarp();
        {  // rows after the last entry's row (every row when the bucket is empty) start at E
            const int last_row = E > 0 ? (int)(key[E - 1] >> cbits) : -1;
            for (int rr = last_row + 1 + lane; rr <= kBkRows; rr += 32) rowb[rr] = (unsigned)E;
        }
        // equal (row, col) keys in COO-position order (duplicates are rare)
        if (__any_sync(0xffffffffu, dup)) {
            for (int p = lane; p + 1 < E; p += 32) {
                if (key[p + 1] != key[p] || (p > 0 && key[p - 1] == key[p])) continue;
                int q = p + 2;
                while (q < E && key[q] == key[p]) ++q;
                for (int i = p + 1; i < q; ++i) {
                    const unsigned v = ord[i];
                    const unsigned kv = rec_in[s0 + (v & kBkWarpIdxMask)].y;  // COO position
                    int j = i - 1;
                    while (j >= p && rec_in[s0 + (ord[j] & kBkWarpIdxMask)].y > kv) {
                        ord[j + 1] = ord[j];
                        --j;
                    }
                    ord[j + 1] = v;
                }
                for (int i = p; i < q; ++i)
                    I.csr_vals[e0 + i] = bk_rec_val(rec_in[s0 + (ord[i] & kBkWarpIdxMask)]);
            }
        }
        __syncwarp();
        for (int r = lane; r <= nr; r += 32) {
            if (r < nr) I.row_ptr[r0 + r] = e0 + rowb[r];
            else if (r0 + nr == I.nrows) I.row_ptr[I.nrows] = I.nnz;
        }
        __syncwarp();
    }
}

// Large buckets (up to 64 rows x 256): one CTA sorts the bucket's keys with a
// block-wide bitonic network in shared memory.  Reads its item count from
// device memory (filled by the warp sort).
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
        __syncthreads();
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// ---- stage 5 ------------------------------------------------------------------
// y[r] = the row's entries summed in column order as one fma chain (the
// reference's sequential row loop, with fused multiply-adds), computed from
// the finished CSR.  Each FP64 warp instruction holds the FP64 pipe for the
// whole warp whatever its active lanes, so one lane per row only pays when
// the 32 rows of a warp instruction have similar lengths: a warp takes a
// 256-row chunk of one instance, counting-sorts its rows by length (256 bins,
// lengths above 255 share the last) in shared memory, and gives each lane one
// row of every group of 32 consecutive rows in that order.  A lane reads its
// row 4 entries at a time with 16-byte loads, ahead of the (in-order) chain.
// Rows above 256 entries are outside the contract and reported.
constexpr int kSpWarps = 8;
constexpr int kSpPerSm = 4;
struct BkSpSmem {
    unsigned cnt[256];
    unsigned start[kSpRows];
    unsigned short len[kSpRows];
    unsigned char order[kSpRows];
};

__global__ void __launch_bounds__(kSpWarps * 32, kSpPerSm)
    bk_spmv_kernel(const BkInst* __restrict__ inst, const BkItem* __restrict__ chunks, unsigned nchunks,
                   unsigned* cursor, unsigned* err) {
    __shared__ BkSpSmem sm_all[kSpWarps];
    const int lane = threadIdx.x & 31;
    BkSpSmem& sm = sm_all[threadIdx.x >> 5];
    bool bad = false;
    for (;;) {
        unsigned it = 0;
        if (lane == 0) it = atomicAdd(cursor, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= nchunks) break;
        const BkItem w = chunks[it];
        const BkInst I = inst[w.inst];
        const long long r0 = (long long)w.tile * kSpRows;
        const int nr = (int)((I.nrows - r0) < kSpRows ? (I.nrows - r0) : kSpRows);
#pragma unroll
        for (int j = 0; j < 8; ++j) sm.cnt[lane + 32 * j] = 0u;
        __syncwarp();
        // row extents, kept inside [0, nnz] whatever the row pointers hold
        for (int i = lane; i < nr; i += 32) {
            long long a = I.row_ptr[r0 + i], e = I.row_ptr[r0 + i + 1];
            a = a < 0 ? 0 : (a > I.nnz ? I.nnz : a);
            e = e < a ? a : (e > I.nnz ? I.nnz : e);
            const long long L = e - a;
            bad |= L > 256;
            const unsigned l = L > 0xFFFF ? 0xFFFFu : (unsigned)L;
            sm.start[i] = (unsigned)a;
            sm.len[i] = (unsigned short)l;
            atomicAdd(&sm.cnt[l > 255u ? 255u : l], 1u);
        }
        __syncwarp();
        {  // exclusive scan of the 256 bin counts; lane l owns bins 8l .. 8l+7
            unsigned c[8], sum = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                c[j] = sm.cnt[8 * lane + j];
                sum += c[j];
            }
            unsigned incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            unsigned run = incl - sum;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                sm.cnt[8 * lane + j] = run;
                run += c[j];
            }
        }
        __syncwarp();
        for (int i = lane; i < nr; i += 32) {
            const unsigned l = sm.len[i];
            sm.order[atomicAdd(&sm.cnt[l > 255u ? 255u : l], 1u)] = (unsigned char)i;
        }
        __syncwarp();
        const int* __restrict__ cols = I.csr_cols;
        const double* __restrict__ vals = I.csr_vals;
        const double* __restrict__ x = I.x;
        const unsigned long long ncols = (unsigned long long)I.ncols;
        for (int g = lane; g < nr; g += 32) {
            const int i = sm.order[g];
            const long long a = sm.start[i];
            const int L = sm.len[i];
            const int* __restrict__ rc = cols + a;
            const double* __restrict__ rv = vals + a;
            double acc = 0.0;
            // x is gathered through L2 only, so that the random x lines do not
            // evict the lanes' sequential row streams
            auto xat = [&](unsigned c) { return c < ncols ? __ldcg(x + c) : 0.0; };
            // entries one at a time until the columns are 16-byte aligned, then
            // 4 per step: the columns by one 16-byte load, the values by two
            // when they are 16-byte aligned too (the parity is fixed per row);
            // the fma chain keeps the row's order throughout
            int k = 0;
            while (k < L && (reinterpret_cast<uintptr_t>(rc + k) & 15)) {
                acc = fma(rv[k], xat((unsigned)rc[k]), acc);
                ++k;
            }
            const bool v16 = (reinterpret_cast<uintptr_t>(rv + k) & 15) == 0;
            for (; k + 4 <= L; k += 4) {
                const int4 c4 = *reinterpret_cast<const int4*>(rc + k);
                double v0, v1, v2, v3;
                if (v16) {
                    const double2 p = *reinterpret_cast<const double2*>(rv + k);
                    const double2 q = *reinterpret_cast<const double2*>(rv + k + 2);
                    v0 = p.x; v1 = p.y; v2 = q.x; v3 = q.y;
                } else {
                    v0 = rv[k]; v1 = rv[k + 1]; v2 = rv[k + 2]; v3 = rv[k + 3];
                }
                const double x0 = xat((unsigned)c4.x), x1 = xat((unsigned)c4.y);
                const double x2 = xat((unsigned)c4.z), x3 = xat((unsigned)c4.w);
                acc = fma(v0, x0, acc);
                acc = fma(v1, x1, acc);
                acc = fma(v2, x2, acc);
                acc = fma(v3, x3, acc);
            }
            for (; k < L; ++k) acc = fma(rv[k], xat((unsigned)rc[k]), acc);
            I.y[r0 + i] = acc;
        }
        __syncwarp();
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
    long long nb_total = 0, entries = 0, nt_total = 0, nc_total = 0;
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
        I.chunk_base = nc_total;
        nt_total += (B.nnz + kTileEntries - 1) / kTileEntries;
        nc_total += (B.nrows + kSpRows - 1) / kSpRows;
        nb_total += I.nbuckets;
        entries += B.nnz;
    }
    if (nb_total >= (1LL << 31) || nt_total >= (1LL << 31) || nc_total >= (1LL << 31) || entries >= (1LL << 32))
        return HYD_CUDA_ERR_UNSUPPORTED;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t inst_b = al(inst.size() * sizeof(BkInst)), tiles_b = al((size_t)nt_total * sizeof(BkItem)),
                 bk_b = al((size_t)nb_total * sizeof(BkItem)), ch_b = al((size_t)nc_total * sizeof(BkItem));
    const size_t cnt_b = al((size_t)nb_total * 4), wide_b = al((size_t)nb_total * 8);
    const size_t vals_b = al((size_t)entries * 8);
    void* buf = nullptr;
    HYD_TRY(device_buffer(d, key, inst_b + tiles_b + 2 * bk_b + ch_b + 2 * cnt_b + 2 * wide_b + vals_b + vals_b + 256,
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
    BkItem* overflow = reinterpret_cast<BkItem*>(take(bk_b));  // buckets above 1536 entries
    BkItem* d_chunks = reinterpret_cast<BkItem*>(take(ch_b));
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
        bk_items_kernel<<<g, 256, 0, s>>>(d_inst, ni, d_tiles, d_bk, d_chunks);
        HYD_TRY(launch_check("bk_items"));
    }
    const size_t n_tiles = (size_t)nt_total, n_buckets = (size_t)nb_total;
    HYD_CUDA_TRY(cudaMemsetAsync(bcount, 0, 2 * cnt_b, s));  // bcount and bfill
    HYD_CUDA_TRY(cudaMemsetAsync(cursors, 0, 64, s));
    const unsigned grid = (unsigned)(d->sm_count * 2);
    if (n_tiles) {
        bk_count_kernel<<<(unsigned)(d->sm_count * kCountPerSm), kBkThreads, 0, s>>>(d_inst, d_tiles,
                                                                                   (unsigned)n_tiles, bcount,
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
    // cursors: 2 the warp sort, 3 the block-wide kernel, 4 the overflow count.
    // (A second warp run over the overflow, with room for 2048 entries, took
    // 0.33 ms against the block-wide kernel's 0.21.)
    {
        auto k1 = bk_bucket_warp_kernel<1536, 5>;
        HYD_TRY(configure_kernel((const void*)k1, d, false));
        k1<<<(unsigned)(d->sm_count * kBkWarpPerSm), 5 * 32, bk_warp_smem<1536, 5>(), s>>>(
            d_inst, d_bk, (unsigned)n_buckets, nullptr, cursors + 2, bstart, bcount, recs, overflow, cursors + 4,
            d->d_err);
        HYD_TRY(launch_check("bk_bucket_warp"));
    }
    HYD_TRY(configure_kernel((const void*)bk_bucket_kernel, d, false));
    bk_bucket_kernel<<<grid, kBkThreads, kBkSmem, s>>>(d_inst, overflow, cursors + 4, cursors + 3, bstart, bcount,
                                                       recs, d->d_err);
    HYD_TRY(launch_check("bk_bucket_large"));
    if (nc_total) {
        bk_spmv_kernel<<<(unsigned)(d->sm_count * kSpPerSm), kSpWarps * 32, 0, s>>>(d_inst, d_chunks,
                                                                                  (unsigned)nc_total, cursors + 5,
                                                                                  d->d_err);
        HYD_TRY(launch_check("bk_spmv"));
    }
    if (!async_tables) HYD_CUDA_TRY(cudaStreamSynchronize(s));
    return HYD_CUDA_OK;
}

size_t batch_pipeline_bucketed_table_bytes(const std::vector<BatchInst>& bi) {
    return (bi.size() * sizeof(BkInst) + 255) & ~(size_t)255;
}

}  // namespace hyd
