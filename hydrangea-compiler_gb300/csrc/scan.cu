// scan.cu -- scan / scan_inclusive / scanr / scanr_inclusive with (+), and
// segmented_reduce (+).
//
// Replaces the serial LoopFold of lowerScanFamily (Lowering.hs:3563-3612; the
// C backend never parallelises a fold, Parallelize.hs:517) and the
// LoopSegRedOuter loop of segmented_reduce (Lowering.hs:874-944,
// `schedule(dynamic)` per CodegenC.hs:1055-1057).
//
// int64: single-pass decoupled look-back (Merrill & Garland, "Single-pass
// Parallel Prefix Scan with Decoupled Look-back", 2016).  Tiles of 4096
// elements take their id from an atomic counter in launch order, so every
// predecessor a tile waits on has already started; a tile publishes its
// aggregate, a warp looks back 32 predecessors at a time, then publishes its
// inclusive prefix.  A tile's status is one 16-byte {flag, value} word
// (TileWord), written and read whole, so a look-back window costs one memory
// round trip.  Every spin is bounded (error bit, no hang).  int64 adds wrap
// and commute, so the result is bit-identical to the serial C fold.  One
// read and one write per element: 16 B/element of HBM traffic.
//
// float64: single pass, deterministic in two levels.  Within a block of 32
// tiles a tile's prefix over its block-mates comes from a fixed warp scan of
// their aggregates; across blocks the block totals are folded left to right
// through the same kind of look-back (lookback_fold).  Every value is defined
// by the data alone, not by timing: results are run-to-run identical.  Within
// a tile the order is fixed too (per-thread serial sums, a fixed shuffle
// tree).  A parallel prefix cannot reproduce the serial fold's roundings; the
// tolerance is |gpu - c| <= 1e-12 * prefix sum of |x| (stated in the tests).
//
// Tiles pass through shared memory padded with one slot per 16 elements, so
// the blocked (8 consecutive elements per thread) and striped accesses are
// free of bank conflicts.
//
// segmented_reduce: tiles of 4096 values (not one warp per segment), so a long
// segment is spread over many CTAs and many short ones share one.  A warp
// finds the tile's segments with a 32-ary search of the offsets; each thread
// keeps segmented running sums of its 8 values and takes the carry of the
// positions before it (one fixed shuffle scan per warp, one over the warps)
// where a segment end needs it; the segment still open at the tile's start
// gets its carry from the predecessors through the deterministic look-back (a
// tile that holds a segment start is an inclusive prefix at once, so the
// look-back stops there).  One read of offsets and values, one write of the
// sums.  Offsets that are not a non-decreasing partition of [0, n_vals] are
// detected by the tiles and handed to a per-segment kernel that gives the
// reference semantics (init, error reported).
//
// Reverse scans read and write index n-1-k for logical position k, exactly the
// ix the reference's lowering computes.
#include "hyd_common.cuh"

namespace hyd {

constexpr int kScanT = 512;
constexpr int kScanIPT = 8;
constexpr int kScanTile = kScanT * kScanIPT;  // 4096 (32 KiB of static shared memory for int64)
constexpr int kScanCtasPerSm = 4;  // resident CTAs per SM (32 registers per thread)
// Tiles sit in shared memory with one 8-byte pad after every 16 elements: a
// thread's blocked run of 8 (stride 64 B between lanes) and the striped
// accesses then both meet no bank conflict.  Unpadded, the blocked accesses
// were 16-way conflicted and the tile copy alone ran at half the copy rate.
constexpr int kScanTileP = kScanTile + kScanTile / 16;
__device__ __forceinline__ int scan_pad(int i) { return i + (i >> 4); }

// --- block-wide exclusive scan of one value per thread (int64, wrapping) ------
template <class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* sh /*[32]*/, T& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? sh[lane] : T(0);
        T wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += y;
        }
        sh[lane] = wi - w;  // exclusive warp offsets
        if (lane == 31) sh[32] = wi;
    }
    __syncthreads();
    total = sh[32];
    T r = sh[warp] + incl - v;
    __syncthreads();
    return r;
}

// The same for float64, without the subtraction the integer form uses for the
// exclusive value (one FP64 operation fewer per thread; the FP64 pipe bounds
// the float64 scan): the exclusive value of a lane is its left neighbour's
// inclusive one.  Fixed order, so run-to-run identical.
template <class T>
__device__ __forceinline__ T block_exclusive_scan_shift(T v, T* sh /*[33]*/, T& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const T y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl = y + incl;
    }
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const T w = lane < nw ? sh[lane] : T(0);
        T wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const T y = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi = y + wi;
        }
        const T wx = __shfl_up_sync(0xffffffffu, wi, 1);
        sh[lane] = lane == 0 ? T(0) : wx;  // exclusive warp offsets
        if (lane == 31) sh[32] = wi;
    }
    __syncthreads();
    total = sh[32];
    const T lx = __shfl_up_sync(0xffffffffu, incl, 1);
    const T r = lane == 0 ? sh[warp] : sh[warp] + lx;
    __syncthreads();
    return r;
}

// Tile load/store in blocked arrangement through shared memory: global
// accesses are coalesced, each thread then owns kScanIPT consecutive logical
// elements.  Logical position k maps to physical index (reverse ? n-1-k : k).
template <class T>
__device__ __forceinline__ void tile_load(const T* in, int64_t n, int64_t base, bool reverse, T* sh,
                                          T (&items)[kScanIPT]) {
    T v[kScanIPT];
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) {  // all loads in flight before the first store
        const int64_t k = base + threadIdx.x + j * kScanT;
        v[j] = k < n ? in[reverse ? (n - 1 - k) : k] : T(0);
    }
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) sh[scan_pad(threadIdx.x + j * kScanT)] = v[j];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) items[j] = sh[scan_pad(threadIdx.x * kScanIPT + j)];
    __syncthreads();
}

template <class T>
__device__ __forceinline__ void tile_store(T* out, int64_t n, int64_t base, bool reverse, T* sh,
                                           const T (&items)[kScanIPT]) {
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) sh[scan_pad(threadIdx.x * kScanIPT + j)] = items[j];
    __syncthreads();
    for (int i = threadIdx.x; i < kScanTile; i += kScanT) {
        const int64_t k = base + i;
        if (k < n) out[reverse ? (n - 1 - k) : k] = sh[scan_pad(i)];
    }
}

// ---- int64 decoupled look-back ----------------------------------------------------
// One TileWord per tile (flag 0 none, 1 aggregate, 2 inclusive prefix).
struct ScanStatus {
    TileWord* word;
    unsigned* tile_counter;
};

__global__ void __launch_bounds__(kScanT, kScanCtasPerSm) scan_i64_lookback_kernel(const long long* __restrict__ in,
                                                                    long long* __restrict__ out, int64_t n,
                                                                    long long init, bool reverse,
                                                                    bool inclusive, ScanStatus st,
                                                                    unsigned* err) {
    __shared__ long long sh_tile[kScanTileP];
    __shared__ long long sh_scan[33];
    __shared__ unsigned sh_tile_id;
    __shared__ long long sh_prefix;
    if (threadIdx.x == 0) sh_tile_id = atomicAdd(st.tile_counter, 1u);
    __syncthreads();
    const unsigned tile = sh_tile_id;
    const int64_t base = (int64_t)tile * kScanTile;

    long long items[kScanIPT];
    tile_load(in, n, base, reverse, sh_tile, items);
    long long tsum = 0;
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) tsum += items[j];
    long long agg;
    const long long texcl = block_exclusive_scan(tsum, sh_scan, agg);

    // publish and look back (warp 0)
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        if (tile == 0) {
            if (lane == 0) {
                tile_word_store(&st.word[0], 2ull, to_bits(init + agg));
                sh_prefix = init;
            }
        } else {
            if (lane == 0) tile_word_store(&st.word[tile], 1ull, to_bits(agg));
            long long running = 0;
            int64_t p = (int64_t)tile - 1;  // window covers p, p-1, ..., p-31
            for (;;) {
                const int64_t q = p - lane;
                // wait until every tile of the window has published something
                unsigned long long bits;
                const unsigned f = lookback_wait_words(st.word, p, lane, bits);
                if (f == 0u) {
                    if (lane == 0) raise_error(err, ERRBIT_TIMEOUT);
                    break;
                }
                const unsigned incl_mask = __ballot_sync(0xffffffffu, f == 2u);
                // nearest predecessor with an inclusive prefix (lowest lane):
                // the aggregates of the lanes before it, then its prefix (before
                // tile 0: the fold's initial value)
                const int stop = incl_mask ? (__ffs(incl_mask) - 1) : 32;
                long long v = 0;
                if (lane <= stop) v = q >= 0 ? from_bits<long long>(bits) : init;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                running += v;
                if (stop < 32) break;
                p -= 32;
            }
            if (lane == 0) {
                tile_word_store(&st.word[tile], 2ull, to_bits(running + agg));
                sh_prefix = running;
            }
        }
    }
    __syncthreads();
    long long acc = sh_prefix + texcl;
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) {
        const long long x = items[j];
        if (inclusive) {
            acc += x;
            items[j] = acc;
        } else {
            items[j] = acc;
            acc += x;
        }
    }
    tile_store(out, n, base, reverse, sh_tile, items);
}

// ---- deterministic decoupled look-back (left fold) -----------------------------------
// One TileWord per tile (flag 0 none, 1 aggregate, 2 inclusive prefix; T's
// bits as the value).
template <class T>
struct FoldStatus {
    TileWord* word;
    unsigned* tile_counter;
    unsigned* bad;  // segmented reduce: the offsets are not a valid partition
};
constexpr int kFoldBuf = 1024;                // aggregates one look-back may collect before it restarts
constexpr unsigned kFoldRestarts = 1u << 12;  // restarts before a look-back gives up

// Warp-wide (all 32 lanes of one warp).  The exclusive prefix of `tile`, as
// the left fold inclusive[s] + aggregate[s+1] + ... + aggregate[tile-1] where s
// is the nearest predecessor that has published an inclusive value (`before`
// stands for the inclusive value of tile -1).  Every inclusive value is made
// the same way, so the result is the left fold of all earlier aggregates,
// whatever the timing.  The fold passes through the inclusive value of every
// tile s+1 .. tile-1 on the way; with kHelp those are published too: a
// predecessor still in its own look-back would compute the same bits, so the
// race is benign, and later tiles find an inclusive value close by (measured:
// it pays for the segmented reduce, whose tiles without a segment start wait
// on long chains, and costs the plain scan 10%).
// Aggregates are collected in sbuf (kFoldBuf); when the nearest inclusive
// predecessor is further back than that, the look-back starts again from
// tile - 1 (nearer prefixes will have appeared by then).  Returns false on
// every lane when a wait ran out.
template <bool kHelp, class T>
__device__ bool lookback_fold(const FoldStatus<T>& st, int64_t tile, T before, T* sbuf, T& prefix) {
    const int lane = threadIdx.x & 31;
    unsigned restarts = 0;
    int64_t p = tile - 1;
    int cnt = 0;
    T base = before;
    for (;;) {
        unsigned long long bits;
        const unsigned f = lookback_wait_words(st.word, p, lane, bits);
        if (f == 0u) return false;
        const int64_t q = p - lane;
        const unsigned incl = __ballot_sync(0xffffffffu, f == 2u);
        const int stop = incl ? __ffs(incl) - 1 : 32;
        if (lane < stop) sbuf[cnt + lane] = from_bits<T>(bits);  // aggregates, nearest first
        if (stop < 32) {
            const T b = q >= 0 ? from_bits<T>(bits) : before;
            base = __shfl_sync(0xffffffffu, b, stop);
            cnt += stop;
            break;
        }
        cnt += 32;
        p -= 32;
        if (cnt + 32 > kFoldBuf) {
            if (++restarts > kFoldRestarts) return false;
            cnt = 0;
            p = tile - 1;
            __nanosleep(256);
        }
    }
    __syncwarp();
    T acc = base;
    if (lane == 0)
        for (int i = cnt - 1; i >= 0; --i) {
            acc = acc + sbuf[i];
            if (kHelp) sbuf[i] = acc;  // the inclusive value of tile - 1 - i
        }
    prefix = __shfl_sync(0xffffffffu, acc, 0);
    if (kHelp) {
        __syncwarp();
        for (int i = lane; i < cnt; i += 32) tile_word_store(&st.word[tile - 1 - i], 2ull, to_bits(sbuf[i]));
    }
    return true;
}

// float64 (and any T) scan, deterministic in two levels.  Tiles form blocks
// of 32 (block k = tiles 32k .. 32k+31):
//  * within a block, tile i's prefix over its block-mates is the value at lane
//    i-1 of a warp inclusive scan (fixed shuffle tree) of the block's tile
//    aggregates, and the block total T(k) is its lane-31 value;
//  * across blocks, B(k) = the left fold of T(0), ..., T(k) onto init, found
//    through lookback_fold over per-block status words (the last tile of a
//    block publishes T(k), then B(k));
//  * the tile's exclusive prefix is B(k-1) + (its within-block prefix).
// Every value is defined by the data alone, not by timing, so results are
// run-to-run identical.  A single-level left fold over tile aggregates puts
// one dependent FP64 add per tile on the scan's critical path (about 76
// cycles each on this part: 1.3 ms at 2^27); here the dependent chain is one
// add per block of 32 tiles.
template <class T>
__global__ void __launch_bounds__(kScanT, kScanCtasPerSm) scan_fold_kernel(const T* __restrict__ in, T* __restrict__ out, int64_t n,
                                                            T init, bool reverse, bool inclusive, FoldStatus<T> st,
                                                            FoldStatus<T> bst, unsigned* err) {
    __shared__ T sh_tile[kScanTileP];
    __shared__ T sh_scan[33];
    __shared__ T sh_fold[kFoldBuf];
    __shared__ unsigned sh_tile_id;
    __shared__ T sh_prefix;
    if (threadIdx.x == 0) sh_tile_id = atomicAdd(st.tile_counter, 1u);
    __syncthreads();
    const unsigned tile = sh_tile_id;
    const int64_t base = (int64_t)tile * kScanTile;
    T items[kScanIPT];
    tile_load(in, n, base, reverse, sh_tile, items);
    // the thread's running sums, in place: items[j] = x_0 + ... + x_j
#pragma unroll
    for (int j = 1; j < kScanIPT; ++j) items[j] = items[j - 1] + items[j];
    T agg;
    const T texcl = block_exclusive_scan_shift(items[kScanIPT - 1], sh_scan, agg);
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const int64_t blk = tile >> 5;
        const int pos = (int)(tile & 31u);
        if (lane == 0) tile_word_store(&st.word[tile], 1ull, to_bits(agg));
        // the aggregates of the block's tiles before this one (earlier tickets)
        unsigned long long f = 1ull, bits = 0ull;
        if (lane < pos) tile_word_load(&st.word[(blk << 5) + lane], f, bits);
        unsigned spins = 0;
        bool ok = true;
        while (__any_sync(0xffffffffu, f == 0ull)) {
            if (++spins > kSpinLimit) {
                ok = false;
                break;
            }
            if (f == 0ull) tile_word_load(&st.word[(blk << 5) + lane], f, bits);
        }
        if (!ok && lane == 0) raise_error(err, ERRBIT_TIMEOUT);
        T sc = lane < pos ? from_bits<T>(bits) : (lane == pos ? agg : T(0));
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const T y = __shfl_up_sync(0xffffffffu, sc, d);
            if (lane >= d) sc = y + sc;
        }
        const T within = __shfl_sync(0xffffffffu, sc, pos > 0 ? pos - 1 : 0);
        const T total = __shfl_sync(0xffffffffu, sc, 31);
        if (pos == 31 && lane == 0) tile_word_store(&bst.word[blk], 1ull, to_bits(total));
        T before = init;  // B(blk - 1)
        if (!lookback_fold<false>(bst, blk, init, sh_fold, before) && lane == 0) raise_error(err, ERRBIT_TIMEOUT);
        if (pos == 31 && lane == 0) tile_word_store(&bst.word[blk], 2ull, to_bits(before + total));
        if (lane == 0) sh_prefix = pos == 0 ? before : before + within;
    }
    __syncthreads();
    // outputs: the thread's prefix plus its running sums (one addition each)
    const T p = sh_prefix + texcl;
    if (inclusive) {
#pragma unroll
        for (int j = 0; j < kScanIPT; ++j) items[j] = p + items[j];
    } else {
#pragma unroll
        for (int j = kScanIPT - 1; j > 0; --j) items[j] = p + items[j - 1];
        items[0] = p;
    }
    tile_store(out, n, base, reverse, sh_tile, items);
}

// ---- segmented reduce over tiles of values ----------------------------------------------
// First index i in [lo, hi) with a[i] >= key (a non-decreasing), else hi.
// Warp-wide: 32 probes per round narrow the range 33-fold, about six dependent
// loads for 2^27 offsets.  Monotone in `key` even for unsorted `a` (a larger
// key never ends left of a smaller one), so tiles' ranges never overlap.
__device__ __forceinline__ int64_t warp_lower_bound(const int64_t* a, int64_t lo, int64_t hi, int64_t key) {
    const int lane = threadIdx.x & 31;
    while (hi - lo > 32) {
        const int64_t span = hi - lo;
        const int64_t p = lo + span * (lane + 1) / 33;  // strictly inside (lo, hi), increasing in lane
        const unsigned m = __ballot_sync(0xffffffffu, a[p] < key);
        const int k = __popc(m);
        const int64_t nlo = k ? lo + span * k / 33 + 1 : lo;
        const int64_t nhi = k < 32 ? lo + span * (k + 1) / 33 : hi;
        lo = nlo;
        hi = nhi;
    }
    const bool below = lo + lane < hi && a[lo + lane] < key;
    return lo + __popc(__ballot_sync(0xffffffffu, below));
}

// (head, value) pairs of a segmented scan: combine(a, b) = (a.h | b.h, b.h ? b.v : a.v + b.v).
template <class T>
__device__ __forceinline__ void seg_combine(bool& h, T& v, bool h_before, T v_before) {
    if (!h) v = v_before + v;
    h = h || h_before;
}

template <class T>
__global__ void __launch_bounds__(kScanT, kScanCtasPerSm) segreduce_tile_kernel(const int64_t* __restrict__ offsets, int64_t nseg,
                                                                 const T* __restrict__ vals, int64_t n_vals, T init,
                                                                 T* __restrict__ out, FoldStatus<T> st,
                                                                 int64_t ntiles, unsigned* err) {
    __shared__ T sh_run[kScanTileP];  // the tile's values, then the running segment sums (padded)
    __shared__ unsigned sh_head[kScanTile / 32];
    __shared__ T sh_fold[kFoldBuf];
    __shared__ T sh_wv[32];             // each warp's inclusive (head seen, sum)
    __shared__ unsigned sh_wh[32];
    __shared__ T sh_wxv[32];            // each warp's exclusive prefix over the warps before it
    __shared__ unsigned sh_wxh[32];
    __shared__ int64_t sh_sb, sh_se;
    __shared__ unsigned sh_tile_id;
    __shared__ T sh_carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) sh_tile_id = atomicAdd(st.tile_counter, 1u);
    if (threadIdx.x < kScanTile / 32) sh_head[threadIdx.x] = 0u;
    __syncthreads();
    const int64_t tile = sh_tile_id;
    const int64_t v0 = tile * kScanTile;
    const int cnt = (int)(n_vals - v0 < kScanTile ? n_vals - v0 : kScanTile);  // >= 0
    const bool last = tile == ntiles - 1;
    // the segments starting in this tile: [sb, se)
    if (warp == 0) {
        const int64_t sb = tile == 0 ? 0 : warp_lower_bound(offsets, 0, nseg, v0);
        if (lane == 0) sh_sb = sb;
    } else if (warp == 1) {
        const int64_t se = last ? nseg : warp_lower_bound(offsets, 0, nseg, v0 + kScanTile);
        if (lane == 0) sh_se = se;
    }
    {
        T v[kScanIPT];
#pragma unroll
        for (int j = 0; j < kScanIPT; ++j) {
            const int i = threadIdx.x + j * kScanT;
            v[j] = i < cnt ? vals[v0 + i] : T(0);
        }
#pragma unroll
        for (int j = 0; j < kScanIPT; ++j) sh_run[scan_pad(threadIdx.x + j * kScanT)] = v[j];
    }
    __syncthreads();
    const int64_t sb = sh_sb, se = sh_se;
    // head flags; every (offsets[s], offsets[s + 1]) pair of this tile's range is checked
    bool bad = se < sb;
    for (int64_t s = sb + threadIdx.x; s < se; s += kScanT) {
        const int64_t o = offsets[s], e = offsets[s + 1];
        const bool ok = o >= v0 && (last ? o <= n_vals : o < v0 + kScanTile) && e >= o && e <= n_vals;
        bad |= !ok;
        if (ok && o - v0 < cnt) atomicOr(&sh_head[(o - v0) >> 5], 1u << ((o - v0) & 31));
    }
    if (threadIdx.x == 0) {
        // the end of the last segment, when values outside every segment
        // follow it here, is a head too: every segment end is then followed
        // by a head or by the end of the tile, which the running sums below rely on
        const int64_t oe = offsets[nseg];
        if (oe >= v0 && oe < v0 + cnt) atomicOr(&sh_head[(oe - v0) >> 5], 1u << ((oe - v0) & 31));
    }
    // the segment open at the tile's start (begun in an earlier tile) ends at offsets[sb]
    const int64_t end_open = sb <= nseg ? offsets[sb] : 0;
    const bool open = tile > 0 && sb > 0 && end_open > v0;
    bad |= sb > nseg || (open && (end_open < v0 || end_open > n_vals));
    if (__syncthreads_or(bad)) {
        if (threadIdx.x == 0) {
            atomicOr(st.bad, 1u);
            // successors must not wait; the per-segment pass redoes every sum
            tile_word_store(&st.word[tile], 2ull, to_bits(T(0)));
        }
        return;
    }
    // segmented scan of the tile: thread t owns positions 8t .. 8t+7.  Only
    // segment ends (and the tile's last value) are read back, so each thread
    // keeps its own segmented running sums (a head restarts the sum) and
    // adds the carry from the positions before it once, at the one position
    // that needs it: the last valid one before its first head.
    const int p0 = threadIdx.x * kScanIPT;
    const unsigned hb = (sh_head[p0 >> 5] >> (p0 & 31)) & 0xffu;
    T x[kScanIPT];
#pragma unroll
    for (int j = 0; j < kScanIPT; ++j) x[j] = sh_run[scan_pad(p0 + j)];
#pragma unroll
    for (int j = 1; j < kScanIPT; ++j)
        if (!((hb >> j) & 1u)) x[j] = x[j - 1] + x[j];
    const bool h = hb != 0u;
    // inclusive warp scan of the threads' (head seen, sum) pairs
    bool hi_ = h;
    T vi = x[kScanIPT - 1];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const bool hu = __shfl_up_sync(0xffffffffu, hi_, d);
        const T vu = __shfl_up_sync(0xffffffffu, vi, d);
        if (lane >= d) seg_combine(hi_, vi, hu, vu);
    }
    if (lane == 31) {
        sh_wv[warp] = vi;
        sh_wh[warp] = hi_;
    }
    __syncthreads();
    if (warp == 0) {
        // exclusive scan over the warps' pairs, once (a fixed shuffle tree)
        constexpr int kW = kScanT / 32;
        bool hw = lane < kW ? sh_wh[lane] != 0u : false;
        T vw = lane < kW ? sh_wv[lane] : T(0);
#pragma unroll
        for (int d = 1; d < kW; d <<= 1) {
            const bool hu = __shfl_up_sync(0xffffffffu, hw, d);
            const T vu = __shfl_up_sync(0xffffffffu, vw, d);
            if (lane >= d) seg_combine(hw, vw, hu, vu);
        }
        const bool hx = __shfl_up_sync(0xffffffffu, hw, 1);
        const T vx = __shfl_up_sync(0xffffffffu, vw, 1);
        if (lane < kW) {
            sh_wxh[lane] = lane > 0 && hx;
            sh_wxv[lane] = lane > 0 ? vx : T(0);
        }
    }
    __syncthreads();
    // this thread's exclusive carry: the warps before, then the lanes before
    bool he = sh_wxh[warp] != 0u;
    T ve = sh_wxv[warp];
    {
        const bool hl = __shfl_up_sync(0xffffffffu, hi_, 1);
        const T vl = __shfl_up_sync(0xffffffffu, vi, 1);
        if (lane > 0) {
            bool hh = hl;
            T vv = vl;
            seg_combine(hh, vv, he, ve);
            he = hh;
            ve = vv;
        }
    }
    {
        const int lim = cnt - p0 < kScanIPT ? (cnt - p0 > 0 ? cnt - p0 : 0) : kScanIPT;
        const int fh = hb ? __ffs(hb) - 1 : kScanIPT;
        const int fix = (fh < lim ? fh : lim) - 1;  // -1: nothing before the first head
        T sel = T(0);
#pragma unroll
        for (int j = 0; j < kScanIPT; ++j)
            if (j == fix) sel = x[j];
        const T fixed = ve + sel;
#pragma unroll
        for (int j = 0; j < kScanIPT; ++j) sh_run[scan_pad(p0 + j)] = j == fix ? fixed : x[j];
    }
    const bool any_head = __syncthreads_or(h);
    // publish and look back (warp 0)
    if (warp == 0) {
        const T tail = cnt > 0 ? sh_run[scan_pad(cnt - 1)] : T(0);
        if (lane == 0) tile_word_store(&st.word[tile], (any_head || !open) ? 2ull : 1ull, to_bits(tail));
        T carry = T(0);
        if (open) {
            if (!lookback_fold<true>(st, tile, T(0), sh_fold, carry) && lane == 0) raise_error(err, ERRBIT_TIMEOUT);
            if (lane == 0 && !any_head) tile_word_store(&st.word[tile], 2ull, to_bits(carry + tail));
        }
        if (lane == 0) sh_carry = carry;
    }
    __syncthreads();
    if (open && end_open <= v0 + cnt && threadIdx.x == 0)
        out[sb - 1] = init + (sh_carry + sh_run[scan_pad((int)(end_open - 1 - v0))]);
    for (int64_t s = sb + threadIdx.x; s < se; s += kScanT) {
        const int64_t o = offsets[s], e = offsets[s + 1];
        if (e == o) out[s] = init;
        else if (e <= v0 + cnt) out[s] = init + sh_run[scan_pad((int)(e - 1 - v0))];
    }
}

// ---- segmented reduce for offsets that are not a valid partition -------------------
// One warp per segment, each segment checked on its own: a segment outside
// [0, n_vals] or with decreasing offsets yields init and is reported.  It runs
// only when the tile kernel found the offsets invalid (*bad != 0) and then
// rewrites every output.
template <class T>
__global__ void __launch_bounds__(256) segreduce_warp_kernel(const int64_t* __restrict__ offsets, int64_t nseg,
                                                             const T* __restrict__ vals, int64_t n_vals, T init,
                                                             T* __restrict__ out, const unsigned* invalid,
                                                             unsigned* err) {
    if (*(volatile const unsigned*)invalid == 0u) return;
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    bool bad = false;
    for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nseg; s += warps) {
        const int64_t start = offsets[s], stop = offsets[s + 1];
        T acc = T(0);
        if (start < 0 || stop > n_vals || stop < start) {
            bad = true;
        } else {
            for (int64_t k = start + lane; k < stop; k += 32) acc += vals[k];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) out[s] = init + acc;
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

}  // namespace hyd

using namespace hyd;

namespace hyd {
// Scratch bytes the decoupled look-back needs for n elements.
size_t scan_i64_scratch_bytes(int64_t n) {
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    return sizeof(TileWord) * (size_t)ntiles + 256;  // + room to align the words to 16 bytes
}

// int64 scan with caller-provided status scratch (scan_i64_scratch_bytes(n))
// and a 4-byte tile counter; both are reset here on the stream.
int scan_i64_launch_with(const long long* in, long long* out, int64_t n, long long init, bool reverse,
                         bool inclusive, void* status_scratch, unsigned* tile_counter, cudaStream_t stream) {
    if (n == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    ScanStatus st;
    st.word = reinterpret_cast<TileWord*>((reinterpret_cast<uintptr_t>(status_scratch) + 15) & ~(uintptr_t)15);
    st.tile_counter = tile_counter;
    HYD_CUDA_TRY(cudaMemsetAsync(st.word, 0, sizeof(TileWord) * (size_t)ntiles, stream));
    HYD_CUDA_TRY(cudaMemsetAsync(st.tile_counter, 0, 4, stream));
    scan_i64_lookback_kernel<<<(unsigned)ntiles, kScanT, 0, stream>>>(in, out, n, init, reverse, inclusive, st,
                                                                       d->d_err);
    return launch_check("scan_i64");
}

// Same, with scratch from the stream's workspace.
int scan_i64_launch(const long long* in, long long* out, int64_t n, long long init, bool reverse,
                    bool inclusive, cudaStream_t stream) {
    if (n == 0) return HYD_CUDA_OK;
    unsigned* counters = nullptr;
    void* scratch = nullptr;
    HYD_TRY(workspace(stream, scan_i64_scratch_bytes(n), &counters, &scratch));
    return scan_i64_launch_with(in, out, n, init, reverse, inclusive, scratch, counters + 8, stream);
}
}  // namespace hyd

extern "C" int hyd_cuda_scan_i64(const int64_t* in, int64_t* out, int64_t n, int64_t init, int reverse,
                                 int inclusive, void* stream) {
    HYD_CHECK_ARG(n >= 0, "scan_i64: negative length");
    HYD_CHECK_ARG(n == 0 || (in != nullptr && out != nullptr), "scan_i64: null buffer");
    HYD_CHECK_ARG(n <= (int64_t)kScanTile * 0x7fffffffLL, "scan_i64: too long");
    return scan_i64_launch(reinterpret_cast<const long long*>(in), reinterpret_cast<long long*>(out), n, init,
                           reverse != 0, inclusive != 0, as_stream(stream));
}

// Status scratch of the left-fold look-back for `ntiles` tiles of (at most)
// 8-byte values: [0, 256) the tile counter (+0) and the invalid-offsets word
// (+4), then `ntiles` tile words and, when `bst` is given, one word per block
// of 32 tiles; all of it zeroed on the stream (one memset).
template <class T>
static int fold_status(cudaStream_t s, int64_t ntiles, FoldStatus<T>* st, FoldStatus<T>* bst = nullptr) {
    static_assert(sizeof(T) <= 8, "a tile word holds a value of at most 8 bytes");
    const int64_t nblocks = bst ? (ntiles + 31) / 32 : 0;
    const size_t bytes = 256 + sizeof(TileWord) * (size_t)(ntiles + nblocks);
    void* scratch = nullptr;
    HYD_TRY(workspace(s, bytes, nullptr, &scratch));
    unsigned char* b = static_cast<unsigned char*>(scratch);  // 256-byte aligned
    st->tile_counter = reinterpret_cast<unsigned*>(b);
    st->bad = reinterpret_cast<unsigned*>(b + 4);
    st->word = reinterpret_cast<TileWord*>(b + 256);
    if (bst) {
        *bst = *st;
        bst->word = st->word + ntiles;
    }
    HYD_CUDA_TRY(cudaMemsetAsync(b, 0, bytes, s));
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_scan_f64(const double* in, double* out, int64_t n, double init, int reverse,
                                 int inclusive, void* stream) {
    HYD_CHECK_ARG(n >= 0, "scan_f64: negative length");
    HYD_CHECK_ARG(n == 0 || (in != nullptr && out != nullptr), "scan_f64: null buffer");
    if (n == 0) return HYD_CUDA_OK;
    cudaStream_t s = as_stream(stream);
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    HYD_CHECK_ARG(ntiles <= 0x7fffffffLL, "scan_f64: too long");
    Device* d = nullptr;
    HYD_TRY(device(&d));
    FoldStatus<double> st, bst;
    HYD_TRY(fold_status(s, ntiles, &st, &bst));
    scan_fold_kernel<double><<<(unsigned)ntiles, kScanT, 0, s>>>(in, out, n, init, reverse != 0, inclusive != 0, st,
                                                                 bst, d->d_err);
    return launch_check("scan_f64");
}

template <class T>
static int segreduce_launch(const int64_t* offsets, int64_t n_offsets, const T* vals, int64_t n_vals, T init,
                            T* out, void* stream, const char* what) {
    HYD_CHECK_ARG(n_offsets >= 1, "%s: need at least one offset", what);
    HYD_CHECK_ARG(offsets != nullptr, "%s: null offsets", what);
    HYD_CHECK_ARG(n_vals >= 0 && (n_vals == 0 || vals != nullptr), "%s: bad values", what);
    const int64_t nseg = n_offsets - 1;
    HYD_CHECK_ARG(nseg == 0 || out != nullptr, "%s: null output", what);
    if (nseg == 0) return HYD_CUDA_OK;
    const int64_t ntiles = n_vals == 0 ? 1 : (n_vals + kScanTile - 1) / kScanTile;
    HYD_CHECK_ARG(ntiles <= 0x7fffffffLL, "%s: too many values", what);
    Device* d = nullptr;
    HYD_TRY(device(&d));
    cudaStream_t s = as_stream(stream);
    FoldStatus<T> st;
    HYD_TRY(fold_status(s, ntiles, &st));
    segreduce_tile_kernel<T><<<(unsigned)ntiles, kScanT, 0, s>>>(offsets, nseg, vals, n_vals, init, out, st, ntiles,
                                                                  d->d_err);
    HYD_TRY(launch_check(what));
    int64_t blocks = (nseg + 7) / 8;
    const int64_t cap = (int64_t)d->sm_count * 8;
    if (blocks > cap) blocks = cap;
    segreduce_warp_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(offsets, nseg, vals, n_vals, init, out, st.bad,
                                                              d->d_err);
    return launch_check(what);
}

extern "C" int hyd_cuda_segmented_reduce_i64(const int64_t* offsets, int64_t n_offsets, const int64_t* vals,
                                             int64_t n_vals, int64_t init, int64_t* out, void* stream) {
    return segreduce_launch<long long>(offsets, n_offsets, reinterpret_cast<const long long*>(vals), n_vals,
                                       (long long)init, reinterpret_cast<long long*>(out), stream,
                                       "segmented_reduce_i64");
}

extern "C" int hyd_cuda_segmented_reduce_f64(const int64_t* offsets, int64_t n_offsets, const double* vals,
                                             int64_t n_vals, double init, double* out, void* stream) {
    return segreduce_launch<double>(offsets, n_offsets, vals, n_vals, init, out, stream, "segmented_reduce_f64");
}
