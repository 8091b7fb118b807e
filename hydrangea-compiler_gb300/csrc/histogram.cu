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

static int plan_hist(const Device* d, long long bins, int strategy, bool packable, HistPlan* p) {
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
        if (tuned >= HYD_SCATTER_SMEM_WARP && tuned <= HYD_SCATTER_GLOBAL &&
            (tuned != HYD_SCATTER_CLUSTER || packable))
            strategy = tuned;
    }
    if (strategy == HYD_SCATTER_AUTO) {
        if (bytes * 4 <= half) {
            strategy = HYD_SCATTER_SMEM_WARP;
        } else if (bytes <= optin) {
            strategy = HYD_SCATTER_SMEM_BLOCK;
        } else {
            // Measured on GB300 (B=65536, 2^27 elements): L2 atomics 0.84 ms,
            // cluster pull 2.5 ms (per-lane DSMEM loads run at ~0.17/clk/SM).
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
static int hist_launch(const Src& src, int64_t n, bool vec, long long bins, u64* hist, int strategy,
                       cudaStream_t stream, const char* what) {
    Device* d = nullptr;
    HYD_TRY(device(&d));
    HistPlan p;
    HYD_TRY(plan_hist(d, bins, strategy, Src::kPackable, &p));
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
    HYD_CHECK_ARG(strategy >= HYD_SCATTER_AUTO && strategy <= HYD_SCATTER_GLOBAL,
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

extern "C" int hyd_cuda_scatter_add_i64(const int64_t* idx, const int64_t* vals, int64_t n,
                                        int64_t* dst, int64_t dst_n, int strategy, void* stream) {
    HYD_CHECK_ARG(n >= 0, "scatter_add_i64: negative length");
    HYD_CHECK_ARG(dst_n > 0, "scatter_add_i64: empty destination");
    HYD_CHECK_ARG(dst != nullptr, "scatter_add_i64: null destination");
    HYD_CHECK_ARG(n == 0 || (idx != nullptr && vals != nullptr), "scatter_add_i64: null input");
    HYD_CHECK_ARG(strategy >= HYD_SCATTER_AUTO && strategy <= HYD_SCATTER_GLOBAL,
                  "scatter_add_i64: unknown strategy %d", strategy);
    HYD_CHECK_ARG(dst_n <= (1LL << 31), "scatter_add_i64: destination beyond 2^31 unsupported");
    if (n == 0) return HYD_CUDA_OK;
    ScatterI64Source src{idx, vals};
    bool vec = ((reinterpret_cast<uintptr_t>(idx) | reinterpret_cast<uintptr_t>(vals)) & 31) == 0;
    return hist_launch(src, n, vec, dst_n, reinterpret_cast<u64*>(dst), strategy, as_stream(stream),
                       "scatter_add_i64");
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
