// histogram.cu -- scatter (+): the fused weighted histogram
//   scatter (+) (fill [B] 0) (map (x % B) data) (map (x * x) data)
// and the unfused scatter-add over materialised routes/values.
//
// Replaces the reference C backend's privatized scatter template
// (CodegenC.hs:1119-1288: an nthreads x B grid of private bins, accumulate,
// merge in thread order) and its atomic template (CodegenC.hs:1084-1118),
// chosen by Parallelize.hs:466-503.  On the GPU the private copies live in
// on-chip memory:
//  * SMEM_WARP   one copy of the B bins per warp (or per group of warps) in
//                shared memory, merged per block into the destination;
//  * SMEM_BLOCK  one copy per block (more bins fit);
//  * CLUSTER     bins spread over the shared memory of a thread-block cluster
//                (2..16 CTAs).  Each round every CTA counting-sorts its tile of
//                elements by owning CTA (warp ballots, no atomics), a cluster
//                barrier publishes the tiles, and each CTA pulls the segments it
//                owns from every peer with distributed-shared-memory loads and
//                applies them locally.  Tiles are double-buffered and the next
//                round's input is prefetched into registers, so one cluster
//                barrier per round is the only synchronisation;
//  * GLOBAL      `red.global.add` straight into the destination (L2 atomics).
//
// 64-bit accumulation uses two 32-bit shared-memory limbs: the low limb's
// atomicAdd returns the old value, whose wrap gives the carry into the high
// limb, and the high limb wraps mod 2^32.  That is exactly int64 wrap-around
// addition, and 32-bit shared atomics run at full rate on sm_103a where 64-bit
// ones do not.  Integer adds commute, so every strategy is bit-identical to the
// C backend.  The input is streamed once with 256-bit non-allocating loads;
// that read is the roofline (8 bytes per element).
#include <cstdlib>
#include <cstring>

#include "hyd_common.cuh"

namespace hyd {

constexpr int kHistThreads = 512;
typedef unsigned long long u64;

// ---- element sources ----------------------------------------------------------
// raw(): the word(s) read for one element; route(): its (bin, value).
// Fused weighted histogram: route x % bins (C truncating remainder), value x*x.
// kPow2: bins is a power of two, so a non-negative x routes by a mask; a
// negative x (whose C remainder is negative, i.e. out of range unless it is 0)
// takes the general path.
template <bool kPow2>
struct WeightedHistSourceT {
    const int64_t* data;
    DivMod64 dm;
    static constexpr bool kPackable = true;  // one 64-bit word per element
    // the bin of a non-negative x is its low word masked (bins <= 2^31)
    static constexpr bool kMaskRoute = kPow2;
    __device__ __forceinline__ unsigned mask32() const { return (unsigned)dm.mask; }
    // Branch-free for a power of two: the masked value is the bin of every
    // non-negative x; a negative x has C remainder -((-x) & mask), which is in
    // range only when it is 0, i.e. exactly when x & mask == 0.  An out-of-range
    // route is returned as -1.
    __device__ __forceinline__ void route(u64 x, long long& bin, u64& val) const {
        if (kPow2) {
            const long long m = (long long)(x & dm.mask);
            bin = ((long long)x >= 0 || m == 0) ? m : -1LL;
        } else {
            bin = dm.rem((long long)x);
        }
        val = x * x;
    }
    __device__ __forceinline__ void one(int64_t i, long long& bin, u64& val) const {
        route((u64)data[i], bin, val);
    }
    // Routes of four elements; true when all four are in [0, bins).  For a
    // power of two the only way out of range is a negative x, so one test of the
    // four sign bits replaces four per-element checks.
    __device__ __forceinline__ bool four(int64_t v, long long bins, long long bin[4], u64 val[4]) const {
        u64x4 q = ldg_stream_u64x4(data + 4 * v);
        const u64 x[4] = {q.x, q.y, q.z, q.w};
        if (kPow2) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                bin[k] = (long long)(x[k] & dm.mask);
                val[k] = x[k] * x[k];
            }
            if ((long long)(x[0] | x[1] | x[2] | x[3]) >= 0) return true;
#pragma unroll
            for (int k = 0; k < 4; ++k) route(x[k], bin[k], val[k]);
            return false;
        }
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            route(x[k], bin[k], val[k]);
            ok &= (unsigned long long)bin[k] < (unsigned long long)bins;
        }
        return ok;
    }
    __device__ __forceinline__ u64x4 raw4(int64_t v) const { return ldg_stream_u64x4(data + 4 * v); }
    __device__ __forceinline__ u64 raw1(int64_t i) const { return (u64)data[i]; }
};

struct ScatterI64Source {
    const int64_t* idx;
    const int64_t* vals;
    static constexpr bool kPackable = false;
    static constexpr bool kMaskRoute = false;
    __device__ __forceinline__ unsigned mask32() const { return 0u; }
    __device__ __forceinline__ void one(int64_t i, long long& bin, u64& val) const {
        bin = idx[i];
        val = (u64)vals[i];
    }
    __device__ __forceinline__ bool four(int64_t v, long long bins, long long bin[4], u64 val[4]) const {
        u64x4 a = ldg_stream_u64x4(idx + 4 * v);
        u64x4 b = ldg_stream_u64x4(vals + 4 * v);
        bin[0] = (long long)a.x; bin[1] = (long long)a.y; bin[2] = (long long)a.z; bin[3] = (long long)a.w;
        val[0] = b.x; val[1] = b.y; val[2] = b.z; val[3] = b.w;
        return ((a.x | a.y | a.z | a.w) < (u64)bins) ||
               ((a.x < (u64)bins) && (a.y < (u64)bins) && (a.z < (u64)bins) && (a.w < (u64)bins));
    }
    // unused (not packable)
    __device__ __forceinline__ void route(u64, long long& bin, u64& val) const { bin = -1; val = 0; }
    __device__ __forceinline__ u64x4 raw4(int64_t) const { return u64x4{0, 0, 0, 0}; }
    __device__ __forceinline__ u64 raw1(int64_t) const { return 0; }
};

// A scatter phase with a guard (Lowering.hs:1768-1790): element i takes part
// only when guard[i] != 0.  Elements left out are routed to bin 0 with the
// value 0, which leaves every sum unchanged, so their index is never checked
// -- the reference does not read it either.
struct GuardedScatterI64Source {
    const int64_t* idx;
    const int64_t* vals;
    const int64_t* guard;
    static constexpr bool kPackable = false;
    static constexpr bool kMaskRoute = false;
    __device__ __forceinline__ unsigned mask32() const { return 0u; }
    __device__ __forceinline__ void one(int64_t i, long long& bin, u64& val) const {
        const bool on = guard[i] != 0;
        bin = on ? idx[i] : 0LL;
        val = on ? (u64)vals[i] : 0ULL;
    }
    __device__ __forceinline__ bool four(int64_t v, long long bins, long long bin[4], u64 val[4]) const {
        const u64x4 g = ldg_stream_u64x4(guard + 4 * v);
        const u64x4 a = ldg_stream_u64x4(idx + 4 * v);
        const u64x4 b = ldg_stream_u64x4(vals + 4 * v);
        bin[0] = g.x ? (long long)a.x : 0LL; bin[1] = g.y ? (long long)a.y : 0LL;
        bin[2] = g.z ? (long long)a.z : 0LL; bin[3] = g.w ? (long long)a.w : 0LL;
        val[0] = g.x ? b.x : 0ULL; val[1] = g.y ? b.y : 0ULL; val[2] = g.z ? b.z : 0ULL; val[3] = g.w ? b.w : 0ULL;
        return ((u64)bin[0] < (u64)bins) && ((u64)bin[1] < (u64)bins) && ((u64)bin[2] < (u64)bins) &&
               ((u64)bin[3] < (u64)bins);
    }
    // unused (not packable)
    __device__ __forceinline__ void route(u64, long long& bin, u64& val) const { bin = -1; val = 0; }
    __device__ __forceinline__ u64x4 raw4(int64_t) const { return u64x4{0, 0, 0, 0}; }
    __device__ __forceinline__ u64 raw1(int64_t) const { return 0; }
};

// Iterate this thread's elements: 32-byte groups t, t+S, ... (two in flight),
// then the scalar remainder.  Groups whose routes are all in range go to
// fast(bin, val) with no per-element check; everything else goes to
// checked(bin, val), which must handle an out-of-range bin.
template <class Src, class F, class FF>
__device__ __forceinline__ void for_each_element(const Src& src, int64_t n, bool vec, long long bins,
                                                 F checked, FF fast) {
    const int64_t S = (int64_t)gridDim.x * blockDim.x;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t tail = 0;
    if (vec) {
        const int64_t nv = n >> 2;
        int64_t v = t;
        for (; v + S < nv; v += 2 * S) {
            long long b0[4], b1[4];
            u64 v0[4], v1[4];
            const bool ok0 = src.four(v, bins, b0, v0);
            const bool ok1 = src.four(v + S, bins, b1, v1);
            if (ok0 && ok1) {
#pragma unroll
                for (int k = 0; k < 4; ++k) fast(b0[k], v0[k]);
#pragma unroll
                for (int k = 0; k < 4; ++k) fast(b1[k], v1[k]);
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) checked(b0[k], v0[k]);
#pragma unroll
                for (int k = 0; k < 4; ++k) checked(b1[k], v1[k]);
            }
        }
        if (v < nv) {
            long long b0[4];
            u64 v0[4];
            src.four(v, bins, b0, v0);
#pragma unroll
            for (int k = 0; k < 4; ++k) checked(b0[k], v0[k]);
        }
        tail = nv * 4;
    }
    for (int64_t i = tail + t; i < n; i += S) {
        long long b;
        u64 v;
        src.one(i, b, v);
        checked(b, v);
    }
}

// Exact 64-bit add into a bin held as two 32-bit shared-memory limbs.
__device__ __forceinline__ void limb_add(unsigned* lo, unsigned* hi, unsigned b, u64 v) {
    const unsigned l = (unsigned)v;
    unsigned h = (unsigned)(v >> 32);
    const unsigned old = atomicAdd(&lo[b], l);
    h += (old + l < old) ? 1u : 0u;  // carry out of the low limb
    if (h) atomicAdd(&hi[b], h);
}
__device__ __forceinline__ u64 limb_value(const unsigned* lo, const unsigned* hi, int b) {
    return (u64)lo[b] + ((u64)hi[b] << 32);
}

// ---- shared-memory privatized (per-warp-group or per-block copies) -------------
// Layout: copy c holds lo[bins] then hi[bins].
template <class Src>
__global__ void __launch_bounds__(kHistThreads, 2)
    hist_smem_kernel(Src src, int64_t n, bool vec, int bins, int copies,
                     u64* __restrict__ hist, unsigned* err) {
    extern __shared__ unsigned sh_limbs[];
    const int total = copies * bins * 2;
    for (int i = threadIdx.x; i < total; i += blockDim.x) sh_limbs[i] = 0u;
    __syncthreads();
    // each half-warp gets its own copy (while copies last): fewer same-address
    // conflicts inside a warp
    unsigned* lo = sh_limbs + (((threadIdx.x >> 5) * 2 + ((threadIdx.x >> 4) & 1)) % copies) * bins * 2;
    unsigned* hi = lo + bins;
    bool bad = false;
    for_each_element(
        src, n, vec, bins,
        [&](long long b, u64 v) {
            const bool ok = (u64)b < (u64)bins;
            bad |= !ok;
            if (ok) limb_add(lo, hi, (unsigned)b, v);
        },
        [&](long long b, u64 v) { limb_add(lo, hi, (unsigned)b, v); });
    __syncthreads();
    for (int b = threadIdx.x; b < bins; b += blockDim.x) {
        u64 s = 0;
        for (int c = 0; c < copies; ++c) {
            const unsigned* cl = sh_limbs + c * bins * 2;
            s += limb_value(cl, cl + bins, b);
        }
        if (s) atomicAdd(&hist[b], s);
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// ---- cluster all-to-all ---------------------------------------------------------
__device__ __forceinline__ unsigned cluster_ctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned map_shared_rank(unsigned local_addr, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_addr), "r"(rank));
    return r;
}
__device__ __forceinline__ u64 ld_dsmem_u64(unsigned addr) {
    u64 v;
    asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(v) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_dsmem_u32(unsigned addr) {
    unsigned v;
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Shared memory of the pull kernel for a cluster of G with 2^shift bins per CTA.
__host__ __device__ constexpr size_t pull_smem_bytes(int G, int shift, int ept) {
    return ((size_t)8 << shift)                           // lo + hi limbs
           + 2ull * (size_t)kHistThreads * ept * 8        // two tiles of raw words
           + 2ull * (G + 1) * 4                           // segment offsets per tile
           + (size_t)G * (kHistThreads / 32) * 4 + 64;    // per-(owner, warp) offsets
}

template <class Src, int G, int EPT>
__global__ void __launch_bounds__(kHistThreads, 1)
    hist_cluster_pull_kernel(Src src, int64_t n, bool vec, long long bins, int shift, int rounds,
                             u64* __restrict__ hist, unsigned* err) {
    constexpr int T = kHistThreads, W = T / 32, R = T * EPT;
    extern __shared__ __align__(16) unsigned char smem[];
    const int per = 1 << shift;
    unsigned* lo = reinterpret_cast<unsigned*>(smem);
    unsigned* hi = lo + per;
    u64* tile = reinterpret_cast<u64*>(smem + ((size_t)8 << shift));  // [2][R]
    unsigned* seg = reinterpret_cast<unsigned*>(tile + 2 * R);          // [2][G+1]
    unsigned* woff = seg + 2 * (G + 1);                                 // [G][W]

    for (int i = threadIdx.x; i < 2 * per; i += T) lo[i] = 0u;
    const unsigned me = cluster_ctarank();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned ltmask = lanemask_lt();
    const int64_t nctas = gridDim.x;
    bool bad = false;

    // Raw words of this CTA's chunk for round r: element e = chunk*R + 4*(t + T*q) + k.
    auto load_round = [&](int r, u64 (&x)[EPT], unsigned& valid) {
        valid = 0u;
        const int64_t base = ((int64_t)r * nctas + blockIdx.x) * (int64_t)R;
#pragma unroll
        for (int q = 0; q < EPT / 4; ++q) {
            const int64_t e = base + 4LL * (threadIdx.x + (int64_t)T * q);
            if (vec && e + 3 < n) {
                u64x4 w = src.raw4(e >> 2);
                x[4 * q] = w.x; x[4 * q + 1] = w.y; x[4 * q + 2] = w.z; x[4 * q + 3] = w.w;
                valid |= 0xFu << (4 * q);
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (e + k < n) {
                        x[4 * q + k] = src.raw1(e + k);
                        valid |= 1u << (4 * q + k);
                    } else {
                        x[4 * q + k] = 0;
                    }
                }
            }
        }
    };

    u64 cur[EPT];
    unsigned cur_valid = 0;
    if (rounds > 0) load_round(0, cur, cur_valid);
    cluster_sync_all();  // limbs zeroed everywhere before any remote activity

    for (int r = 0; r < rounds; ++r) {
        const int buf = r & 1;
        u64 nxt[EPT];
        unsigned nxt_valid = 0;
        if (r + 1 < rounds) load_round(r + 1, nxt, nxt_valid);  // in flight during this round

        // --- owner of every element, and its rank inside (warp, owner) --------
        unsigned char own[EPT];
        unsigned short pos[EPT];
        unsigned cnt[G];
#pragma unroll
        for (int o = 0; o < G; ++o) cnt[o] = 0u;
#pragma unroll
        for (int j = 0; j < EPT; ++j) {
            bool ok = (cur_valid >> j) & 1u;
            long long b = 0;
            u64 v;
            if (ok) {
                src.route(cur[j], b, v);
                if ((u64)b >= (u64)bins) {
                    bad = true;
                    ok = false;
                }
            }
            const unsigned o = ok ? (unsigned)(b >> shift) : 0xFFu;
            own[j] = (unsigned char)o;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const unsigned m = __ballot_sync(0xffffffffu, o == (unsigned)g);
                if (o == (unsigned)g) pos[j] = (unsigned short)(cnt[g] + __popc(m & ltmask));
                cnt[g] += __popc(m);
            }
        }
        if (lane < G) {
            unsigned c = 0;
#pragma unroll
            for (int g = 0; g < G; ++g)
                if (g == lane) c = cnt[g];
            woff[lane * W + warp] = c;
        }
        __syncthreads();
        // exclusive scan over (owner-major, warp-minor) counts by warp 0
        if (warp == 0) {
            constexpr int PER_LANE = (G * W + 31) / 32;
            unsigned vals[PER_LANE];
            unsigned s = 0;
#pragma unroll
            for (int k = 0; k < PER_LANE; ++k) {
                const int idx = lane * PER_LANE + k;
                vals[k] = idx < G * W ? woff[idx] : 0u;
                s += vals[k];
            }
            unsigned incl = s;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += y;
            }
            unsigned run = incl - s;
#pragma unroll
            for (int k = 0; k < PER_LANE; ++k) {
                const int idx = lane * PER_LANE + k;
                if (idx < G * W) {
                    if ((idx % W) == 0) seg[buf * (G + 1) + idx / W] = run;
                    woff[idx] = run;
                }
                run += vals[k];
            }
            if (lane == 31) seg[buf * (G + 1) + G] = incl;
        }
        __syncthreads();
        u64* t = tile + buf * R;
#pragma unroll
        for (int j = 0; j < EPT; ++j)
            if (own[j] != 0xFFu) t[woff[own[j] * W + warp] + pos[j]] = cur[j];

        cluster_sync_all();  // every CTA's tile `buf` and offsets are published

        // --- pull my segment from each CTA of the cluster and apply ------------
        const unsigned seg_base = (unsigned)__cvta_generic_to_shared(seg + buf * (G + 1));
        const unsigned tile_base = (unsigned)__cvta_generic_to_shared(t);
        unsigned start[G], len[G];
        unsigned total = 0;
#pragma unroll
        for (int s = 0; s < G; ++s) {
            const unsigned sb = map_shared_rank(seg_base, (unsigned)s);
            const unsigned a = ld_dsmem_u32(sb + 4u * me);
            const unsigned b = ld_dsmem_u32(sb + 4u * (me + 1));
            start[s] = a;
            len[s] = b - a;
            total += b - a;
        }
        // four independent DSMEM loads in flight per thread; consecutive lanes
        // read consecutive words of the same segment (coalesced)
        for (unsigned q0 = threadIdx.x; q0 < total; q0 += 4 * T) {
            u64 xs[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const unsigned q = q0 + u * T;
                xs[u] = 0;
                if (q < total) {
                    unsigned rem = q, rank = 0;
#pragma unroll
                    for (int s = 0; s < G - 1; ++s) {
                        if (rank == (unsigned)s && rem >= len[s]) {
                            rem -= len[s];
                            rank = s + 1;
                        }
                    }
                    unsigned st = 0;
#pragma unroll
                    for (int s = 0; s < G; ++s)
                        if (rank == (unsigned)s) st = start[s];
                    xs[u] = ld_dsmem_u64(map_shared_rank(tile_base + 8u * (st + rem), rank));
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (q0 + u * T < total) {
                    long long b;
                    u64 v;
                    src.route(xs[u], b, v);
                    limb_add(lo, hi, (unsigned)(b & (per - 1)), v);
                }
            }
        }

#pragma unroll
        for (int j = 0; j < EPT; ++j) cur[j] = nxt[j];
        cur_valid = nxt_valid;
    }
    cluster_sync_all();  // no peer reads this CTA's tiles any more
    const long long first = (long long)me << shift;
    for (int i = threadIdx.x; i < per; i += T) {
        const long long g = first + i;
        const u64 s = limb_value(lo, hi, i);
        if (g < bins && s) atomicAdd(&hist[g], s);
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// ---- partition: a staging pass, then one shared-memory pass per bin range -----
// For bins beyond one SM's shared memory.  Pass 1 reads the data once and
// writes every tile of kPartTile elements back, in place in a staging buffer,
// with its elements grouped by bin range (range = bin >> kPartShift) and the
// P + 1 run boundaries of the tile in a table.  Pass 2 is a persistent kernel
// over (range, chunk of tiles) work items taken in range order: a CTA keeps
// the 2^kPartShift bins of its current range as 32-bit limbs in shared memory,
// reads only that range's run of each tile, and flushes the limbs to the
// histogram with global atomics when it moves to another range.  Per element:
// one word read, written and read again, and shared-memory atomics, instead
// of one L2 atomic.  Integer sums are exact, so the order inside a run is
// immaterial.
constexpr int kPartThreads = 512;
constexpr int kPartEPT = 8;
constexpr int kPartTile = kPartThreads * kPartEPT;  // 4096 elements
constexpr int kPartWarps = kPartThreads / 32;
constexpr int kPartMaxRanges = 32;
constexpr int kPartShift = 14;  // 16384 bins (128 KB of limbs) per range
// three tile buffers (bulk-loaded, grouped in place, bulk-stored) + mbarriers
constexpr int kPartBufs = 3;
constexpr int kPartCtasPerSm = 2;
constexpr size_t kPartStageSmem = kPartBufs * (size_t)kPartTile * 8 + 8 * kPartBufs;
constexpr int kApplyThreads = 1024;
constexpr int kApplyUnroll = 8;
constexpr int64_t kPartMaxStage = (int64_t)1 << 27;  // elements staged per round
constexpr int64_t kPartAutoMin = (int64_t)1 << 23;   // AUTO picks the partition from here
// queue words after the stream's counter base: [0] finished apply CTAs,
// [32 + r] elements of range r; the last apply CTA to finish zeroes them for
// the next round
constexpr int kPartQueueWord = 64;

// Pass 1.  Tiles stream through three shared-memory buffers: one thread
// bulk-loads tile i + 2 while tile i is grouped (mbarrier completion, bounded
// waits), and the grouped tile is bulk-stored from the same buffer.  The load
// of tile i + 2 goes into the buffer of tile i - 1 and is issued at the end of
// iteration i, right after tile i's store: by then the store of tile i - 1 has
// long read its buffer, so the wait for that never holds up the block.  Every
// thread counts its eight elements per range in packed 16-bit fields (NW words
// of two ranges); one block-wide exclusive scan of those words gives each
// thread its offset inside every range; the elements, held in registers, are
// then written back into the buffer they were read from in range order.
template <class Src, int NW>
__global__ void __launch_bounds__(kPartThreads, kPartCtasPerSm)
    hist_part_stage_kernel(Src src, const int64_t n, const bool bulk, const long long bins, const int P,
                           const int64_t ntiles, u64* __restrict__ staged, unsigned short* __restrict__ bounds,
                           unsigned* __restrict__ counts, unsigned* err) {
    extern __shared__ __align__(128) unsigned char part_smem[];
    u64* inbuf = reinterpret_cast<u64*>(part_smem);
    const unsigned in0 = (unsigned)__cvta_generic_to_shared(inbuf);
    const unsigned bar0 = in0 + kPartBufs * kPartTile * 8;
    __shared__ unsigned wtot[NW][kPartWarps];
    __shared__ unsigned rstart[kPartMaxRanges + 1];
    __shared__ unsigned scur[NW == 2 ? 4 * kPartThreads : 1];  // per-thread range cursors
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool bad = false;
    if (threadIdx.x == 0) {
        for (int q = 0; q < kPartBufs; ++q) mbar_init(bar0 + 8 * q, 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    // bytes of tile t that come in bulk: its whole 16-byte units
    auto bulk_bytes = [&](int64_t t) -> unsigned {
        const int64_t cnt = n - t * kPartTile < kPartTile ? n - t * kPartTile : kPartTile;
        return bulk ? (unsigned)((cnt * 8) & ~(int64_t)15) : 0u;
    };
    auto issue = [&](int64_t t, int buf) {
        const unsigned bytes = bulk_bytes(t);
        mbar_expect_tx(bar0 + 8 * buf, bytes);
        if (bytes) bulk_load_1d(in0 + buf * kPartTile * 8, src.data + t * kPartTile, bytes, bar0 + 8 * buf);
    };
    if (threadIdx.x == 0)
        for (int q = 0; q < kPartBufs - 1; ++q)
            if (blockIdx.x + (int64_t)q * gridDim.x < ntiles) issue(blockIdx.x + (int64_t)q * gridDim.x, q);
    int64_t tile = blockIdx.x;
    unsigned it = 0;
    bool timed_out = false;
    for (; tile < ntiles; tile += gridDim.x, ++it) {
        const int buf = (int)(it % kPartBufs);
        // one thread polls (acquire on the mbarrier phase); the block barrier
        // then orders the landed tile before every thread's reads
        const bool arrived = threadIdx.x == 0 ? mbar_wait_bounded(bar0 + 8 * buf, (it / kPartBufs) & 1u) : true;
        if (__syncthreads_or(!arrived)) {
            timed_out = true;
            break;
        }
        const int64_t e0 = tile * kPartTile;
        const int cnt = (int)(n - e0 < kPartTile ? n - e0 : kPartTile);
        const int have = (int)(bulk_bytes(tile) / 8);
        u64* const in = inbuf + buf * kPartTile;
        u64 x[kPartEPT];
        int r[kPartEPT];  // range; -1: no element or out of range
        // a full tile in shared memory whose elements all route by the mask
        // ("clean") needs no per-element presence or range checks
        const bool full = have == kPartTile;
        unsigned hi_or = 0u;  // high words: all zero -> staged as 4-byte records
        bool fast = false;
        // thread t holds elements 2(t + q kPartThreads) + {0, 1}, q < 4: each
        // 16-byte load of a warp covers 512 consecutive bytes (no bank
        // conflict); which thread holds an element does not matter, the
        // elements of a range only need distinct slots of its run
        if (full) {
            const ulonglong2* in2 = reinterpret_cast<const ulonglong2*>(in);
#pragma unroll
            for (int q = 0; q < kPartEPT / 2; ++q) {
                const ulonglong2 a = in2[threadIdx.x + q * kPartThreads];
                x[2 * q] = a.x;
                x[2 * q + 1] = a.y;
            }
#pragma unroll
            for (int k = 0; k < kPartEPT; ++k) {
                hi_or |= (unsigned)(x[k] >> 32);
                r[k] = 0;
            }
            if constexpr (Src::kMaskRoute) {
                if ((int)hi_or >= 0) {
                    fast = true;
                    const unsigned m = src.mask32();
#pragma unroll
                    for (int k = 0; k < kPartEPT; ++k) r[k] = (int)(((unsigned)x[k] & m) >> kPartShift);
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < kPartEPT; ++k) {
                const int j = 2 * (threadIdx.x + (k >> 1) * kPartThreads) + (k & 1);
                r[k] = j < cnt ? 0 : -1;
                x[k] = j < have ? in[j] : (j < cnt ? src.raw1(e0 + j) : 0ULL);
            }
#pragma unroll
            for (int k = 0; k < kPartEPT; ++k) hi_or |= r[k] == 0 ? (unsigned)(x[k] >> 32) : 0u;
            if constexpr (Src::kMaskRoute) {
                if ((int)hi_or >= 0) {
                    fast = true;
                    const unsigned m = src.mask32();
#pragma unroll
                    for (int k = 0; k < kPartEPT; ++k)
                        if (r[k] == 0) r[k] = (int)(((unsigned)x[k] & m) >> kPartShift);
                }
            }
        }
        if (!fast) {
#pragma unroll
            for (int k = 0; k < kPartEPT; ++k) {
                if (r[k] == 0) {
                    long long b;
                    u64 v;
                    src.route(x[k], b, v);
                    const bool valid = (u64)b < (u64)bins;
                    bad |= !valid;
                    r[k] = valid ? (int)(b >> kPartShift) : -1;
                }
            }
        }
        const bool clean = full && fast;
        // per-thread counts, two 16-bit fields per word (ranges 2w and 2w + 1)
        unsigned C[NW];
        if constexpr (NW == 2) {
            // up to four ranges: count in one word of 8-bit fields, then widen
            unsigned c8 = 0u;
            if (clean) {
#pragma unroll
                for (int k = 0; k < kPartEPT; ++k) c8 += 1u << (r[k] << 3);
            } else {
#pragma unroll
                for (int k = 0; k < kPartEPT; ++k)
                    if (r[k] >= 0) c8 += 1u << (r[k] << 3);
            }
            C[0] = (c8 & 0xffu) | ((c8 & 0xff00u) << 8);
            C[1] = ((c8 >> 16) & 0xffu) | ((c8 >> 8) & 0xff0000u);
        } else {
#pragma unroll
            for (int w = 0; w < NW; ++w) C[w] = 0u;
#pragma unroll
            for (int k = 0; k < kPartEPT; ++k) {
                if (r[k] >= 0) {
                    const unsigned one = 1u << ((r[k] & 1) << 4);
                    // masked adds: no per-element indexing into C (which would
                    // move it to local memory)
#pragma unroll
                    for (int w = 0; w < NW; ++w) C[w] += one & (0u - (unsigned)((r[k] >> 1) == w));
                }
            }
        }
        // block-wide exclusive scan of the packed counts (fields never carry:
        // a range holds at most kPartTile < 2^16 elements of a tile)
        unsigned E[NW];
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            unsigned inc = C[w];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += y;
            }
            E[w] = inc - C[w];
            if (lane == 31) wtot[w][warp] = inc;
        }
        const bool wide = __syncthreads_or(hi_or != 0u);
        if (warp == 0) {
            // warp totals -> exclusive warp offsets per word; lane q < P picks
            // up the tile's count of range q, then the range starts are scanned
            unsigned tq = 0u;
#pragma unroll
            for (int w = 0; w < NW; ++w) {
                const unsigned t0 = lane < kPartWarps ? wtot[w][lane] : 0u;
                unsigned inc = t0;
#pragma unroll
                for (int o = 1; o < kPartWarps; o <<= 1) {
                    const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += y;
                }
                const unsigned tot = __shfl_sync(0xffffffffu, inc, kPartWarps - 1);
                if (lane < kPartWarps) wtot[w][lane] = inc - t0;
                if ((lane >> 1) == w) tq = (tot >> ((lane & 1) << 4)) & 0xffffu;
            }
            if (lane >= P) tq = 0u;
            unsigned inc = tq;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += y;
            }
            if (lane < P) {
                rstart[lane] = inc - tq;
                if (tq) atomicAdd(&counts[lane], tq);
            }
            if (lane == P - 1) rstart[P] = inc;
        }
        __syncthreads();
#pragma unroll
        for (int w = 0; w < NW; ++w) E[w] += wtot[w][warp];
        if constexpr (NW == 2) {
            // this thread's next slot in each range, as a shared-memory cursor
            // (cursor q of thread t at cur[q * kPartThreads + t]: conflict-free)
            unsigned* cur = scur + threadIdx.x;
            cur[0] = rstart[0] + (E[0] & 0xffffu);
            cur[kPartThreads] = rstart[1] + (E[0] >> 16);
            cur[2 * kPartThreads] = rstart[2] + (E[1] & 0xffffu);
            cur[3 * kPartThreads] = rstart[3] + (E[1] >> 16);
            unsigned* in32 = reinterpret_cast<unsigned*>(in);
            auto place = [&](int k) {
                unsigned* c = cur + r[k] * kPartThreads;
                const unsigned p = *c;
                *c = p + 1u;
                if (wide) in[p] = x[k];
                else in32[p] = (unsigned)x[k];
            };
            if (clean) {
#pragma unroll
                for (int k = 0; k < kPartEPT; ++k) place(k);
            } else {
#pragma unroll
                for (int k = 0; k < kPartEPT; ++k)
                    if (r[k] >= 0) place(k);
            }
        } else {
#pragma unroll
            for (int k = 0; k < kPartEPT; ++k) {
                if (r[k] >= 0) {
                    const int sh = (r[k] & 1) << 4;
                    unsigned e = 0u;
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        const unsigned sel = 0u - (unsigned)((r[k] >> 1) == w);
                        e |= E[w] & sel;
                        E[w] += (1u << sh) & sel;
                    }
                    const unsigned slot = rstart[r[k]] + ((e >> sh) & 0xffffu);
                    if (wide) in[slot] = x[k];
                    else reinterpret_cast<unsigned*>(in)[slot] = (unsigned)x[k];
                }
            }
        }
        // generic-proxy writes, then the bulk store reads the buffer
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            const unsigned esz = wide ? 8u : 4u;
            const unsigned all = rstart[P] * esz;
            const unsigned sbytes = all & ~15u;
            if (sbytes)
                asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(staged + e0),
                             "r"(in0 + buf * kPartTile * 8), "r"(sbytes)
                             : "memory");
            // one group per tile, empty or not, so that "all groups but the
            // newest" below always means the stores of tiles before this one
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            // the last partial 16 bytes
            unsigned char* dst = reinterpret_cast<unsigned char*>(staged + e0);
            const unsigned char* srcb = reinterpret_cast<const unsigned char*>(in);
            for (unsigned bb = sbytes; bb < all; bb += 4)
                *reinterpret_cast<unsigned*>(dst + bb) = *reinterpret_cast<const unsigned*>(srcb + bb);
            // tile i + 2 into the buffer of tile i - 1, whose store has read it
            const int64_t ahead = tile + (int64_t)(kPartBufs - 1) * gridDim.x;
            if (ahead < ntiles) {
                asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(ahead, (int)((it + kPartBufs - 1) % kPartBufs));
            }
        }
        // run bounds; bit 15 marks a tile staged as 4-byte records
        if (threadIdx.x <= P)
            bounds[tile * (P + 1) + threadIdx.x] = (unsigned short)(rstart[threadIdx.x] | (wide ? 0u : 0x8000u));
    }
    if (timed_out && threadIdx.x == 0) {
        // let the loads in flight (tiles i and i + 1) land before the shared
        // memory is released
        for (int q = 0; q < kPartBufs - 1; ++q)
            if (tile + (int64_t)q * gridDim.x < ntiles)
                mbar_wait_bounded(bar0 + 8 * ((it + q) % kPartBufs), ((it + q) / kPartBufs) & 1u);
        raise_error(err, ERRBIT_TIMEOUT);
    }
    if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// Pass 2.  Each CTA takes one range -- ranges get CTAs in proportion to their
// element counts, at least one each when non-empty -- and an equal share of
// the tiles; the run bounds of up to kApplyChunk tiles at a time are staged in
// shared memory, and warp w reads the runs of tiles w, w + 32, ... with
// kApplyUnroll loads in flight per lane.  The limbs are flushed once, at the end.
constexpr int kApplyChunk = 1024;

template <class Src>
__global__ void __launch_bounds__(kApplyThreads, 1)
    hist_part_apply_kernel(Src src, const long long bins, const int P, const int64_t ntiles,
                           const u64* __restrict__ staged, const unsigned short* __restrict__ bounds,
                           unsigned* __restrict__ queue, u64* __restrict__ hist) {
    extern __shared__ __align__(16) unsigned part_limbs[];
    constexpr int per = 1 << kPartShift;
    unsigned* lo = part_limbs;
    unsigned* hi = part_limbs + per;
    __shared__ int s_range, s_index, s_share;
    __shared__ unsigned s_run[kApplyChunk];  // start | end << 16
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < 2 * per; i += kApplyThreads) part_limbs[i] = 0u;
    if (threadIdx.x == 0) {
        const volatile unsigned* cnt = queue + 32;
        long long total = 0;
        int nonempty = 0;
        for (int r = 0; r < P; ++r) {
            total += cnt[r];
            nonempty += cnt[r] != 0u;
        }
        int range = -1, index = 0, share = 0;
        if (total > 0) {
            const long long spare = (long long)gridDim.x - nonempty;
            long long cum = 0, first = 0;
            for (int r = 0; r < P; ++r) {
                const long long c = cnt[r];
                if (c == 0) continue;
                const long long a = 1 + spare * (cum + c) / total - spare * cum / total;
                if ((long long)blockIdx.x >= first && (long long)blockIdx.x < first + a) {
                    range = r;
                    index = (int)(blockIdx.x - first);
                    share = (int)a;
                    break;
                }
                first += a;
                cum += c;
            }
        }
        s_range = range;
        s_index = index;
        s_share = share;
    }
    __syncthreads();
    const int range = s_range;
    if (range >= 0) {
        const int64_t t_lo = ntiles * s_index / s_share, t_hi = ntiles * (s_index + 1) / s_share;
        for (int64_t c0 = t_lo; c0 < t_hi; c0 += kApplyChunk) {
            const int nb = (int)(t_hi - c0 < kApplyChunk ? t_hi - c0 : kApplyChunk);
            for (int q = threadIdx.x; q < nb; q += kApplyThreads) {
                const unsigned short* bt = bounds + (c0 + q) * (P + 1) + range;
                s_run[q] = (unsigned)bt[0] | ((unsigned)bt[1] << 16);  // bit 15 of each: 4-byte records
            }
            __syncthreads();
            for (int q = warp; q < nb; q += kApplyThreads / 32) {
                const unsigned se = s_run[q];
                const int s0 = (int)(se & 0x7fffu), e = (int)((se >> 16) & 0x7fffu);
                const u64* run = staged + (c0 + q) * kPartTile;
                auto apply1 = [&](u64 xv) {
                    long long b;
                    u64 v;
                    src.route(xv, b, v);
                    limb_add(lo, hi, (unsigned)(b & (per - 1)), v);
                };
                if (se & 0x8000u) {
                    // 4-byte records: ragged ends one at a time, 16-byte loads between
                    const unsigned* run32 = reinterpret_cast<const unsigned*>(run);
                    const int a0 = (s0 + 3) & ~3, a1 = e & ~3;
                    if (a0 >= a1) {
                        if (lane < e - s0) apply1(run32[s0 + lane]);
                        continue;
                    }
                    if (lane < a0 - s0) apply1(run32[s0 + lane]);
                    if (lane < e - a1) apply1(run32[a1 + lane]);
                    const uint4* p4 = reinterpret_cast<const uint4*>(run32);
                    constexpr int kU4 = Src::kMaskRoute ? kApplyUnroll : kApplyUnroll / 4;
                    for (int i = (a0 >> 2) + lane; i < (a1 >> 2); i += 32 * kU4) {
                        uint4 y[kU4];
#pragma unroll
                        for (int u = 0; u < kU4; ++u)
                            y[u] = i + 32 * u < (a1 >> 2) ? p4[i + 32 * u] : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                        for (int u = 0; u < kU4; ++u) {
                            if (i + 32 * u < (a1 >> 2)) {
                                apply1(y[u].x);
                                apply1(y[u].y);
                                apply1(y[u].z);
                                apply1(y[u].w);
                            }
                        }
                    }
                    continue;
                }
                // odd ends one at a time; the pairs in between with 16-byte loads
                const int a0 = (s0 + 1) & ~1, a1 = e & ~1;
                if (lane == 0 && (s0 & 1) && s0 < e) apply1(run[s0]);
                if (lane == 1 && (e & 1) && e - 1 >= a0) apply1(run[e - 1]);
                const ulonglong2* pr = reinterpret_cast<const ulonglong2*>(run);
                // 16-byte loads in flight per lane (fewer for the division route,
                // which needs more registers)
                constexpr int kU = Src::kMaskRoute ? kApplyUnroll : kApplyUnroll / 2;
                for (int i = (a0 >> 1) + lane; i < (a1 >> 1); i += 32 * kU) {
                    ulonglong2 x[kU];
#pragma unroll
                    for (int u = 0; u < kU; ++u)
                        x[u] = i + 32 * u < (a1 >> 1) ? pr[i + 32 * u] : make_ulonglong2(0ULL, 0ULL);
#pragma unroll
                    for (int u = 0; u < kU; ++u) {
                        if (i + 32 * u < (a1 >> 1)) {
                            apply1(x[u].x);
                            apply1(x[u].y);
                        }
                    }
                }
            }
            __syncthreads();
        }
        const long long first = (long long)range << kPartShift;
        for (int i = threadIdx.x; i < per; i += kApplyThreads) {
            const u64 sum = limb_value(lo, hi, i);
            if (sum && first + i < bins) atomicAdd(&hist[first + i], sum);
        }
    }
    // the last CTA to finish zeroes the counts for the next round
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(queue, 1u) == gridDim.x - 1) {
            for (int r = 0; r < P; ++r) queue[32 + r] = 0u;
            queue[0] = 0u;
            __threadfence();
        }
    }
}

// ---- global atomics -----------------------------------------------------------
template <class Src>
__global__ void __launch_bounds__(kHistThreads, 2)
    hist_global_kernel(Src src, int64_t n, bool vec, long long bins, u64* __restrict__ hist,
                       unsigned* err) {
    bool bad = false;
    for_each_element(
        src, n, vec, bins,
        [&](long long b, u64 v) {
            const bool ok = (u64)b < (u64)bins;
            bad |= !ok;
            if (ok && v) atomicAdd(&hist[b], v);
        },
        [&](long long b, u64 v) {
            if (v) atomicAdd(&hist[b], v);
        });
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

// ---- host side -------------------------------------------------------------------
struct HistPlan {
    int strategy;
    int copies;   // SMEM_*: copies per block
    int cluster;  // CLUSTER: CTAs per cluster
    int shift;    // CLUSTER: log2(bins per CTA)
    int ept;      // CLUSTER: elements per thread per round
    size_t smem;  // dynamic shared memory bytes
    int blocks;
};

static int log2_ceil(long long v) {
    int s = 0;
    while ((1LL << s) < v) ++s;
    return s;
}

// Shared memory one CTA may use while keeping 2 CTAs per SM.
static size_t smem_half(const Device* d) { return (size_t)d->max_smem_optin / 2 - 1024; }

static int plan_cluster(const Device* d, long long bins, int G, HistPlan* p) {
    const size_t optin = (size_t)d->max_smem_optin - 1024;
    const int shift = log2_ceil((bins + G - 1) / G);
    for (int ept : {16, 8}) {
        if (pull_smem_bytes(G, shift, ept) <= optin) {
            p->cluster = G;
            p->shift = shift;
            p->ept = ept;
            p->smem = pull_smem_bytes(G, shift, ept);
            p->blocks = (d->sm_count / G) * G;
            return HYD_CUDA_OK;
        }
    }
    return HYD_CUDA_ERR_UNSUPPORTED;
}

static int plan_hist(const Device* d, long long bins, int64_t n, int strategy, bool packable, HistPlan* p) {
    const size_t bytes = (size_t)bins * 8;  // two 32-bit limbs per bin
    const size_t half = smem_half(d);
    const size_t optin = (size_t)d->max_smem_optin - 1024;
    const int warps = kHistThreads / 32;
    p->copies = 1;
    p->cluster = 1;
    p->shift = 0;
    p->ept = 0;
    p->smem = 0;
    if (strategy == HYD_SCATTER_AUTO) {
        const int tuned = tune_lookup_hist(bins);
        if (tuned >= HYD_SCATTER_SMEM_WARP && tuned <= HYD_SCATTER_PARTITION &&
            ((tuned != HYD_SCATTER_CLUSTER && tuned != HYD_SCATTER_PARTITION) || packable))
            strategy = tuned;
    }
    if (strategy == HYD_SCATTER_AUTO) {
        if (bytes * 4 <= half) {
            strategy = HYD_SCATTER_SMEM_WARP;
        } else if (bytes <= optin) {
            strategy = HYD_SCATTER_SMEM_BLOCK;
        } else if (packable && bins <= (4LL << kPartShift) && n >= kPartAutoMin) {
            // Measured on GB300 (B=65536, 2^27 elements): partition 0.58 ms,
            // L2 atomics 0.84 ms, cluster pull 2.5 ms (per-lane DSMEM loads run
            // at ~0.17/clk/SM).  Beyond four ranges, or on small inputs, the L2
            // atomics win.
            strategy = HYD_SCATTER_PARTITION;
        } else {
            strategy = HYD_SCATTER_GLOBAL;
        }
    }
    p->strategy = strategy;
    switch (strategy) {
        case HYD_SCATTER_SMEM_WARP: {
            if (bytes > half)
                return set_error(HYD_CUDA_ERR_UNSUPPORTED, "SMEM_WARP: %lld bins exceed shared memory", bins);
            int c = (int)(half / bytes);
            p->copies = c > 2 * warps ? 2 * warps : c;
            p->smem = bytes * p->copies;
            p->blocks = d->sm_count * 2;
            return HYD_CUDA_OK;
        }
        case HYD_SCATTER_SMEM_BLOCK:
            if (bytes > optin)
                return set_error(HYD_CUDA_ERR_UNSUPPORTED, "SMEM_BLOCK: %lld bins exceed shared memory", bins);
            p->smem = bytes;
            p->blocks = d->sm_count * (bytes <= half ? 2 : 1);
            return HYD_CUDA_OK;
        case HYD_SCATTER_CLUSTER: {
            if (!packable)
                return set_error(HYD_CUDA_ERR_UNSUPPORTED, "CLUSTER: source is not single-word");
            const char* force = getenv("HYD_CUDA_HIST_CLUSTER");  // tuning override "G" or "G:EPT"
            if (force) {
                int G = atoi(force), ept = 0;
                const char* c = strchr(force, ':');
                if (c) ept = atoi(c + 1);
                if ((G == 2 || G == 4 || G == 8 || G == 16) && plan_cluster(d, bins, G, p) == HYD_CUDA_OK) {
                    if (ept == 8 || ept == 16) {
                        p->ept = ept;
                        p->smem = pull_smem_bytes(G, p->shift, ept);
                        if (p->smem > optin) return set_error(HYD_CUDA_ERR_UNSUPPORTED, "CLUSTER override does not fit");
                    }
                    return HYD_CUDA_OK;
                }
            }
            for (int G : {2, 4, 8, 16}) {
                if ((long long)G > bins) break;
                if (plan_cluster(d, bins, G, p) == HYD_CUDA_OK) return HYD_CUDA_OK;
            }
            return set_error(HYD_CUDA_ERR_UNSUPPORTED, "CLUSTER: %lld bins exceed 16 CTAs of shared memory", bins);
        }
        case HYD_SCATTER_PARTITION: {
            if (!packable)
                return set_error(HYD_CUDA_ERR_UNSUPPORTED, "PARTITION: source is not single-word");
            const long long P = (bins + (1LL << kPartShift) - 1) >> kPartShift;
            if (P > kPartMaxRanges)
                return set_error(HYD_CUDA_ERR_UNSUPPORTED, "PARTITION: %lld bins exceed %d ranges", bins,
                                 kPartMaxRanges);
            p->cluster = (int)P;
            p->smem = (size_t)8 << kPartShift;
            if (p->smem > optin) return set_error(HYD_CUDA_ERR_UNSUPPORTED, "PARTITION: shared memory too small");
            p->blocks = d->sm_count;
            return HYD_CUDA_OK;
        }
        case HYD_SCATTER_GLOBAL:
            p->blocks = d->sm_count * 2;
            return HYD_CUDA_OK;
        default:
            return set_error(HYD_CUDA_ERR_INVALID, "unknown scatter strategy %d", strategy);
    }
}

// Raise a kernel's dynamic shared memory limit to the device maximum, once per
// (kernel, device).
template <class K>
static int allow_max_smem(K k, const Device* d, bool nonportable_cluster = false) {
    return hyd::configure_kernel((const void*)k, d, nonportable_cluster);
}

template <class Src, int G, int EPT>
static int launch_pull(const Src& src, int64_t n, bool vec, long long bins, const HistPlan& p, u64* hist,
                       const Device* d, cudaStream_t stream) {
    unsigned* err = d->d_err;
    auto k = hist_cluster_pull_kernel<Src, G, EPT>;
    HYD_TRY(allow_max_smem(k, d, G > 8));
    const int64_t R = (int64_t)kHistThreads * EPT;
    const int64_t per_round = R * p.blocks;
    const int rounds = (int)((n + per_round - 1) / per_round);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)p.blocks);
    cfg.blockDim = dim3(kHistThreads);
    cfg.dynamicSmemBytes = p.smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    HYD_CUDA_TRY(cudaLaunchKernelEx(&cfg, k, src, n, vec, bins, p.shift, rounds, hist, err));
    return HYD_CUDA_OK;
}

template <class Src>
static int launch_cluster(const Src& src, int64_t n, bool vec, long long bins, const HistPlan& p, u64* hist,
                          const Device* err, cudaStream_t stream) {
    if constexpr (Src::kPackable) {
        switch (p.cluster * 100 + p.ept) {
            case 216: return launch_pull<Src, 2, 16>(src, n, vec, bins, p, hist, err, stream);
            case 208: return launch_pull<Src, 2, 8>(src, n, vec, bins, p, hist, err, stream);
            case 416: return launch_pull<Src, 4, 16>(src, n, vec, bins, p, hist, err, stream);
            case 408: return launch_pull<Src, 4, 8>(src, n, vec, bins, p, hist, err, stream);
            case 816: return launch_pull<Src, 8, 16>(src, n, vec, bins, p, hist, err, stream);
            case 808: return launch_pull<Src, 8, 8>(src, n, vec, bins, p, hist, err, stream);
            case 1616: return launch_pull<Src, 16, 16>(src, n, vec, bins, p, hist, err, stream);
            case 1608: return launch_pull<Src, 16, 8>(src, n, vec, bins, p, hist, err, stream);
        }
    }
    return set_error(HYD_CUDA_ERR_UNSUPPORTED, "no cluster kernel for G=%d ept=%d", p.cluster, p.ept);
}

template <class Src>
static int launch_partition(const Src& src, int64_t n, long long bins, const HistPlan& p, u64* hist, Device* d,
                            cudaStream_t stream) {
    if constexpr (Src::kPackable) {
        const int P = p.cluster;
        const int64_t seg = n < kPartMaxStage ? n : kPartMaxStage;
        const int64_t max_tiles = (seg + kPartTile - 1) / kPartTile;
        const size_t stage_bytes = (size_t)max_tiles * kPartTile * 8;
        const size_t bounds_bytes = (size_t)max_tiles * (P + 1) * sizeof(unsigned short);
        unsigned* counters = nullptr;
        void* scratch = nullptr;
        HYD_TRY(workspace(stream, stage_bytes + bounds_bytes, &counters, &scratch));
        u64* staged = static_cast<u64*>(scratch);
        unsigned short* bounds = reinterpret_cast<unsigned short*>(static_cast<unsigned char*>(scratch) + stage_bytes);
        unsigned* queue = counters + kPartQueueWord;
        auto stage_k = P <= 4 ? hist_part_stage_kernel<Src, 2>
                       : P <= 8 ? hist_part_stage_kernel<Src, 4>
                       : P <= 16 ? hist_part_stage_kernel<Src, 8> : hist_part_stage_kernel<Src, 16>;
        auto apply_k = hist_part_apply_kernel<Src>;
        HYD_TRY(allow_max_smem(stage_k, d));
        HYD_TRY(allow_max_smem(apply_k, d));
        // bulk copies need 16-byte aligned tiles (every tile start is, if the data is)
        const bool bulk = (reinterpret_cast<uintptr_t>(src.data) & 15) == 0;
        for (int64_t off = 0; off < n; off += kPartMaxStage) {
            const int64_t m = n - off < kPartMaxStage ? n - off : kPartMaxStage;
            const int64_t ntiles = (m + kPartTile - 1) / kPartTile;
            Src part = src;
            part.data += off;
            const int64_t g1max = (int64_t)kPartCtasPerSm * d->sm_count;
            const unsigned g1 = (unsigned)(ntiles < g1max ? ntiles : g1max);
            stage_k<<<g1, kPartThreads, kPartStageSmem, stream>>>(part, m, bulk, bins, P, ntiles, staged,
                                                                 bounds, queue + 32, d->d_err);
            HYD_TRY(launch_check("weighted_histogram partition stage"));
            apply_k<<<p.blocks, kApplyThreads, p.smem, stream>>>(part, bins, P, ntiles, staged, bounds, queue, hist);
            HYD_TRY(launch_check("weighted_histogram partition apply"));
        }
        return HYD_CUDA_OK;
    }
    return set_error(HYD_CUDA_ERR_UNSUPPORTED, "PARTITION: source is not single-word");
}

template <class Src>
static int hist_launch(const Src& src, int64_t n, bool vec, long long bins, u64* hist, int strategy,
                       cudaStream_t stream, const char* what) {
    Device* d = nullptr;
    HYD_TRY(device(&d));
    HistPlan p;
    HYD_TRY(plan_hist(d, bins, n, strategy, Src::kPackable, &p));
    const int64_t groups = (n + 3) / 4;
    const int64_t want = (groups + kHistThreads - 1) / kHistThreads;
    switch (p.strategy) {
        case HYD_SCATTER_SMEM_WARP:
        case HYD_SCATTER_SMEM_BLOCK: {
            if (want < p.blocks) p.blocks = want < 1 ? 1 : (int)want;
            auto k = hist_smem_kernel<Src>;
            HYD_TRY(allow_max_smem(k, d));
            k<<<p.blocks, kHistThreads, p.smem, stream>>>(src, n, vec, (int)bins, p.copies, hist, d->d_err);
            break;
        }
        case HYD_SCATTER_CLUSTER:
            HYD_TRY(launch_cluster(src, n, vec, bins, p, hist, d, stream));
            break;
        case HYD_SCATTER_PARTITION:
            HYD_TRY(launch_partition(src, n, bins, p, hist, d, stream));
            break;
        case HYD_SCATTER_GLOBAL:
            if (want < p.blocks) p.blocks = want < 1 ? 1 : (int)want;
            hist_global_kernel<Src><<<p.blocks, kHistThreads, 0, stream>>>(src, n, vec, bins, hist, d->d_err);
            break;
    }
    return launch_check(what);
}

// Plain fp64 scatter-add (global atomics; order-dependent rounding).
__global__ void scatter_add_f64_kernel(const int64_t* __restrict__ idx, const double* __restrict__ vals,
                                       int64_t n, double* dst, int64_t dst_n, unsigned* err) {
    const int64_t S = (int64_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += S) {
        int64_t b = idx[i];
        if ((uint64_t)b < (uint64_t)dst_n) atomicAdd(&dst[b], vals[i]);
        else bad = true;
    }
    if (bad) raise_error(err, ERRBIT_BOUNDS);
}

}  // namespace hyd

using namespace hyd;

extern "C" int hyd_cuda_weighted_histogram_i64(const int64_t* data, int64_t n, int64_t bins,
                                               int64_t* hist, int strategy, void* stream) {
    HYD_CHECK_ARG(n >= 0, "weighted_histogram: negative length %lld", (long long)n);
    HYD_CHECK_ARG(bins > 0, "weighted_histogram: bins must be positive (got %lld)", (long long)bins);
    HYD_CHECK_ARG(hist != nullptr, "weighted_histogram: null histogram");
    HYD_CHECK_ARG(n == 0 || data != nullptr, "weighted_histogram: null data");
    HYD_CHECK_ARG(strategy >= HYD_SCATTER_AUTO && strategy <= HYD_SCATTER_PARTITION,
                  "weighted_histogram: unknown strategy %d", strategy);
    HYD_CHECK_ARG(bins <= (1LL << 31), "weighted_histogram: bins beyond 2^31 unsupported");
    if (n == 0) return HYD_CUDA_OK;
    const bool vec = (reinterpret_cast<uintptr_t>(data) & 31) == 0;
    DivMod64 dm;
    dm.init(bins);
    if (dm.shift >= 0) {
        WeightedHistSourceT<true> src{data, dm};
        return hist_launch(src, n, vec, bins, reinterpret_cast<u64*>(hist), strategy, as_stream(stream),
                           "weighted_histogram_i64");
    }
    WeightedHistSourceT<false> src{data, dm};
    return hist_launch(src, n, vec, bins, reinterpret_cast<u64*>(hist), strategy, as_stream(stream),
                       "weighted_histogram_i64");
}

extern "C" int hyd_cuda_weighted_histogram_plan(int64_t n, int64_t bins, int strategy, int* chosen, int* launches) {
    HYD_CHECK_ARG(n >= 0 && bins > 0 && bins <= (1LL << 31), "weighted_histogram_plan: bad shape");
    HYD_CHECK_ARG(strategy >= HYD_SCATTER_AUTO && strategy <= HYD_SCATTER_PARTITION,
                  "weighted_histogram_plan: unknown strategy %d", strategy);
    Device* d = nullptr;
    HYD_TRY(device(&d));
    HistPlan p;
    HYD_TRY(plan_hist(d, bins, n, strategy, true, &p));
    if (chosen) *chosen = p.strategy;
    if (launches) {
        const int64_t rounds = (n + kPartMaxStage - 1) / kPartMaxStage;
        *launches = n == 0 ? 0 : (p.strategy == HYD_SCATTER_PARTITION ? (int)(2 * rounds) : 1);
    }
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_scatter_add_i64(const int64_t* idx, const int64_t* vals, int64_t n,
                                        int64_t* dst, int64_t dst_n, int strategy, void* stream) {
    HYD_CHECK_ARG(n >= 0, "scatter_add_i64: negative length");
    HYD_CHECK_ARG(dst_n > 0, "scatter_add_i64: empty destination");
    HYD_CHECK_ARG(dst != nullptr, "scatter_add_i64: null destination");
    HYD_CHECK_ARG(n == 0 || (idx != nullptr && vals != nullptr), "scatter_add_i64: null input");
    HYD_CHECK_ARG(strategy >= HYD_SCATTER_AUTO && strategy <= HYD_SCATTER_PARTITION,
                  "scatter_add_i64: unknown strategy %d", strategy);
    HYD_CHECK_ARG(dst_n <= (1LL << 31), "scatter_add_i64: destination beyond 2^31 unsupported");
    if (n == 0) return HYD_CUDA_OK;
    ScatterI64Source src{idx, vals};
    bool vec = ((reinterpret_cast<uintptr_t>(idx) | reinterpret_cast<uintptr_t>(vals)) & 31) == 0;
    return hist_launch(src, n, vec, dst_n, reinterpret_cast<u64*>(dst), strategy, as_stream(stream),
                       "scatter_add_i64");
}

extern "C" int hyd_cuda_scatter_add_guarded_i64(const int64_t* idx, const int64_t* vals, const int64_t* guard,
                                                int64_t n, int64_t* dst, int64_t dst_n, int strategy, void* stream) {
    HYD_CHECK_ARG(n >= 0, "scatter_add_guarded_i64: negative length");
    HYD_CHECK_ARG(dst_n > 0, "scatter_add_guarded_i64: empty destination");
    HYD_CHECK_ARG(dst != nullptr, "scatter_add_guarded_i64: null destination");
    HYD_CHECK_ARG(n == 0 || (idx != nullptr && vals != nullptr && guard != nullptr),
                  "scatter_add_guarded_i64: null input");
    HYD_CHECK_ARG(strategy >= HYD_SCATTER_AUTO && strategy <= HYD_SCATTER_PARTITION,
                  "scatter_add_guarded_i64: unknown strategy %d", strategy);
    HYD_CHECK_ARG(dst_n <= (1LL << 31), "scatter_add_guarded_i64: destination beyond 2^31 unsupported");
    if (n == 0) return HYD_CUDA_OK;
    GuardedScatterI64Source src{idx, vals, guard};
    const bool vec =
        ((reinterpret_cast<uintptr_t>(idx) | reinterpret_cast<uintptr_t>(vals) | reinterpret_cast<uintptr_t>(guard)) &
         31) == 0;
    return hist_launch(src, n, vec, dst_n, reinterpret_cast<u64*>(dst), strategy, as_stream(stream),
                       "scatter_add_guarded_i64");
}

extern "C" int hyd_cuda_scatter_add_f64(const int64_t* idx, const double* vals, int64_t n,
                                        double* dst, int64_t dst_n, void* stream) {
    HYD_CHECK_ARG(n >= 0, "scatter_add_f64: negative length");
    HYD_CHECK_ARG(dst_n > 0 && dst != nullptr, "scatter_add_f64: empty or null destination");
    HYD_CHECK_ARG(n == 0 || (idx != nullptr && vals != nullptr), "scatter_add_f64: null input");
    if (n == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    int64_t want = (n + 255) / 256;
    int blocks = (int)(want < d->sm_count * 4 ? want : d->sm_count * 4);
    scatter_add_f64_kernel<<<blocks, 256, 0, as_stream(stream)>>>(idx, vals, n, dst, dst_n, d->d_err);
    return launch_check("scatter_add_f64");
}
