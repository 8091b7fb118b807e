// serve.cu -- the resident request server: continuous batching of compiled
// kernel invocations of mixed kinds and sizes on one GPU.
//
// The reference has no server; its nearest pieces are the memoised zero-arg
// procedures of the C backend (CodegenC.hs:690-707) and the Metal export
// lifecycle that keeps device buffers between calls (CodegenMSL.hs:1120-1181).
// Here requests reference device-resident arrays and are served by a
// dispatcher thread inside the runtime:
//  * admission: a request is admitted when the working sets of everything in
//    flight plus its own fit the HBM budget (FIFO; a request larger than the
//    whole budget is rejected with HYD_CUDA_ERR_BUDGET);
//  * continuous batching: whenever a launch slot (stream) is free, every
//    admitted waiting request (up to max_batch) is coalesced into one batch:
//    dot / histogram / Laplacian requests into ONE persistent launch that
//    drains a device-side queue of (request, tile) work items, SpMV requests
//    into the batched COO -> CSR -> SpMV pipeline; batches on different slots
//    overlap on the device, and requests arriving meanwhile join the next
//    batch as soon as a slot and memory free up;
//  * completion is stamped by a host function enqueued behind each batch
//    (no polling), so latency = arrival -> result ready.
// Each request's result is computed by the same per-request code whatever it
// is batched with: dot products reduce fixed 2^16-element tiles in a fixed
// order and the last tile combines the partials in tile order; histograms and
// stencils are exact.  So a result is bit-identical alone and in any mix.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <string>
#include <thread>
#include <vector>

#include "batch.cuh"
#include "fp64_emu.cuh"
#include "hyd_common.cuh"

namespace hyd {

constexpr int kMixThreads = 512;
constexpr long long kDotTile = 1LL << 16;
constexpr long long kHistTile = 1LL << 18;
constexpr int kLapTH = 64, kLapTW = 128;
static_assert(kLapTH * kLapTW % kMixThreads == 0 && kMixThreads % kLapTW == 0, "Laplacian tile vs threads");
constexpr int kMixMaxBins = 8192;  // histogram requests served up to this many bins
constexpr size_t kMixSmem = 64 * 1024;

struct MixReq {
    int kind;
    int index;          // position in the batch (status slot)
    long long n, m;
    const void* a;
    const void* b;
    void* out;
    long long item_base;  // first work item
    long long nitems;
    long long scratch;    // first 8-byte word of its partials in the batch scratch
};

__device__ __forceinline__ double lap_body(double a, double b, double c, double d, double e) {
    // a + b + c + d + (e * -4.0), evaluated as the C backend does (4e exact);
    // the first two additions on the integer pipe (exact, FP64 fallback)
    const double t3 = __dadd_rn(dadd_pos(dadd_pos(a, b), c), d);
    return __fma_rn(e, -4.0, t3);
}

__device__ __forceinline__ double block_sum_fixed(double v, double* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (warp == 0) {
        r = lane < (kMixThreads / 32) ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;  // thread 0
}

__device__ __forceinline__ void limb_add32(unsigned* lo, unsigned* hi, unsigned b, unsigned long long v) {
    const unsigned l = (unsigned)v;
    unsigned h = (unsigned)(v >> 32);
    const unsigned old = atomicAdd(&lo[b], l);
    h += (old + l < old) ? 1u : 0u;
    if (h) atomicAdd(&hi[b], h);
}

__global__ void __launch_bounds__(kMixThreads, 2)
    mixed_batch_kernel(const MixReq* __restrict__ reqs, int nreq, long long total_items, unsigned* cursor,
                       unsigned* done, unsigned long long* scratch, int* status) {
    extern __shared__ __align__(16) unsigned char mix_smem[];
    __shared__ double sh_red[32];
    __shared__ unsigned sh_item;
    __shared__ bool sh_last;
    for (;;) {
        if (threadIdx.x == 0) sh_item = atomicAdd(cursor, 1u);
        __syncthreads();
        const long long item = sh_item;
        __syncthreads();
        if (item >= total_items) break;
        int lo = 0, hi = nreq - 1;  // last request with item_base <= item
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (reqs[mid].item_base <= item) lo = mid;
            else hi = mid - 1;
        }
        const MixReq R = reqs[lo];
        const long long tile = item - R.item_base;
        if (R.kind == HYD_REQ_DOT) {
            const double* xs = static_cast<const double*>(R.a);
            const double* ys = static_cast<const double*>(R.b);
            const long long base = tile * kDotTile;
            const long long len = R.n - base < kDotTile ? R.n - base : kDotTile;
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
            const bool vec = ((reinterpret_cast<uintptr_t>(xs) | reinterpret_cast<uintptr_t>(ys)) & 31) == 0;
            long long tail = 0;
            if (vec) {
                const long long nv = len >> 2;
                for (long long v = threadIdx.x; v < nv; v += kMixThreads) {
                    const f64x4 x = ldg_stream_f64x4(xs + base + 4 * v);
                    const f64x4 y = ldg_stream_f64x4(ys + base + 4 * v);
                    a0 = fma(x.x, y.x, a0); a1 = fma(x.y, y.y, a1);
                    a2 = fma(x.z, y.z, a2); a3 = fma(x.w, y.w, a3);
                }
                tail = nv * 4;
            }
            for (long long i = tail + threadIdx.x; i < len; i += kMixThreads) a0 = fma(xs[base + i], ys[base + i], a0);
            const double part = block_sum_fixed((a0 + a1) + (a2 + a3), sh_red);
            if (threadIdx.x == 0) {
                reinterpret_cast<double*>(scratch)[R.scratch + tile] = part;
                __threadfence();
                sh_last = atomicAdd(&done[R.index], 1u) == (unsigned)(R.nitems - 1);
            }
            __syncthreads();
            if (sh_last && threadIdx.x < 32) {
                __threadfence();
                double s = 0.0;
                // L2 loads (the partials were fenced by their writers), all in flight
                const double* p = reinterpret_cast<const double*>(scratch) + R.scratch;
                for (long long t = threadIdx.x; t < R.nitems; t += 32) s += __ldcg(p + t);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (threadIdx.x == 0) *static_cast<double*>(R.out) = s;
            }
        } else if (R.kind == HYD_REQ_HIST) {
            const long long* data = static_cast<const long long*>(R.a);
            const int bins = (int)R.m;
            // copies of the bins in shared memory: one per warp while they fit
            int copies = (int)(kMixSmem / ((size_t)bins * 8));
            if (copies > kMixThreads / 32) copies = kMixThreads / 32;
            unsigned* limbs = reinterpret_cast<unsigned*>(mix_smem);
            for (int i = threadIdx.x; i < copies * bins * 2; i += kMixThreads) limbs[i] = 0u;
            __syncthreads();
            unsigned* lo_l = limbs + ((threadIdx.x >> 5) % copies) * bins * 2;
            unsigned* hi_l = lo_l + bins;
            const bool pow2 = (bins & (bins - 1)) == 0;
            const long long base = tile * kHistTile;
            const long long len = R.n - base < kHistTile ? R.n - base : kHistTile;
            bool bad = false;
            auto add1 = [&](long long x) {
                const long long b = pow2 ? ((x >= 0 || (x & (bins - 1)) == 0) ? (x & (bins - 1)) : -1) : x % bins;
                if ((unsigned long long)b < (unsigned long long)bins)
                    limb_add32(lo_l, hi_l, (unsigned)b, (unsigned long long)x * (unsigned long long)x);
                else
                    bad = true;
            };
            long long tail = 0;
            if ((reinterpret_cast<uintptr_t>(data + base) & 31) == 0) {  // 32-byte vectors, two in flight
                const long long nv = len >> 2;
                long long v = threadIdx.x;
                for (; v + kMixThreads < nv; v += 2 * kMixThreads) {
                    const u64x4 q0 = ldg_stream_u64x4(reinterpret_cast<const unsigned long long*>(data + base) + 4 * v);
                    const u64x4 q1 = ldg_stream_u64x4(reinterpret_cast<const unsigned long long*>(data + base) +
                                                      4 * (v + kMixThreads));
                    add1((long long)q0.x); add1((long long)q0.y); add1((long long)q0.z); add1((long long)q0.w);
                    add1((long long)q1.x); add1((long long)q1.y); add1((long long)q1.z); add1((long long)q1.w);
                }
                for (; v < nv; v += kMixThreads) {
                    const u64x4 q = ldg_stream_u64x4(reinterpret_cast<const unsigned long long*>(data + base) + 4 * v);
                    add1((long long)q.x); add1((long long)q.y); add1((long long)q.z); add1((long long)q.w);
                }
                tail = nv * 4;
            }
            for (long long i = tail + threadIdx.x; i < len; i += kMixThreads) add1(data[base + i]);
            if (bad) status[R.index] = HYD_CUDA_ERR_BOUNDS;
            __syncthreads();
            unsigned long long* part = scratch + R.scratch + tile * (long long)bins;
            for (int b = threadIdx.x; b < bins; b += kMixThreads) {
                unsigned long long s = 0;
                for (int c = 0; c < copies; ++c) {
                    const unsigned* cl = limbs + c * bins * 2;
                    s += (unsigned long long)cl[b] + ((unsigned long long)cl[bins + b] << 32);
                }
                part[b] = s;
            }
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) sh_last = atomicAdd(&done[R.index], 1u) == (unsigned)(R.nitems - 1);
            __syncthreads();
            if (sh_last) {
                __threadfence();
                // L2 loads (the partials were fenced by their writers), four in flight
                const unsigned long long* p = scratch + R.scratch;
                unsigned long long* out = static_cast<unsigned long long*>(R.out);
                for (int b = threadIdx.x; b < bins; b += kMixThreads) {
                    unsigned long long s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                    long long t = 0;
                    for (; t + 3 < R.nitems; t += 4) {
                        s0 += __ldcg(p + t * bins + b);
                        s1 += __ldcg(p + (t + 1) * bins + b);
                        s2 += __ldcg(p + (t + 2) * bins + b);
                        s3 += __ldcg(p + (t + 3) * bins + b);
                    }
                    for (; t < R.nitems; ++t) s0 += __ldcg(p + t * bins + b);
                    out[b] = (s0 + s1) + (s2 + s3);  // integer sums: order-free
                }
            }
            __syncthreads();  // shared bins are reused by the next item
        } else {  // HYD_REQ_LAPLACIAN, one clamp step
            // a thread sweeps kRowsPer rows of one column, carrying the rows
            // above and at the point in registers: three loads per point
            const double* in = static_cast<const double*>(R.a);
            double* out = static_cast<double*>(R.out);
            const long long h = R.n, w = R.m;
            const long long ntj = (w + kLapTW - 1) / kLapTW;
            const long long i0 = (tile / ntj) * kLapTH, j0 = (tile % ntj) * kLapTW;
            constexpr int kRowsPer = kLapTH * kLapTW / kMixThreads;
            const long long j = j0 + (threadIdx.x % kLapTW);
            const long long ib = i0 + (threadIdx.x / kLapTW) * kRowsPer;
            if (j < w && ib < h) {
                const long long jm = j > 0 ? j - 1 : 0, jp = j + 1 < w ? j + 1 : w - 1;
                double up = in[(ib > 0 ? ib - 1 : 0) * w + j];
                double mid = in[ib * w + j];
#pragma unroll
                for (int k = 0; k < kRowsPer; ++k) {
                    const long long i = ib + k;
                    if (i >= h) break;
                    const double dn = in[(i + 1 < h ? i + 1 : h - 1) * w + j];
                    const double* row = in + i * w;
                    out[i * w + j] = lap_body(up, dn, row[jm], row[jp], mid);
                    up = mid;
                    mid = dn;
                }
            }
        }
    }
}

// ---------------------------------------------------------------- helpers
static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static int validate(const hyd_request_t& r) {
    switch (r.kind) {
        case HYD_REQ_DOT:
            if (r.n < 0 || (r.n > 0 && (!r.in0 || !r.in1)) || !r.out0) return HYD_CUDA_ERR_INVALID;
            return HYD_CUDA_OK;
        case HYD_REQ_HIST:
            if (r.n < 0 || r.m < 1 || (r.n > 0 && !r.in0) || !r.out0) return HYD_CUDA_ERR_INVALID;
            if (r.m > kMixMaxBins) return HYD_CUDA_ERR_UNSUPPORTED;
            return HYD_CUDA_OK;
        case HYD_REQ_LAPLACIAN:
            if (r.n < 1 || r.m < 1 || !r.in0 || !r.out0 || r.in0 == r.out0) return HYD_CUDA_ERR_INVALID;
            return HYD_CUDA_OK;
        case HYD_REQ_SPMV:
            if (r.n < 1 || r.n >= (1LL << 31) || r.m < 0 || !r.in3 || !r.out0 || !r.out1 ||
                (r.m > 0 && (!r.in0 || !r.in1 || !r.in2 || !r.out2 || !r.out3)))
                return HYD_CUDA_ERR_INVALID;
            return HYD_CUDA_OK;
        default:
            return HYD_CUDA_ERR_INVALID;
    }
}

static long long working_set(const hyd_request_t& r) {
    switch (r.kind) {
        case HYD_REQ_DOT: return 16 * r.n + 8;
        case HYD_REQ_HIST: return 8 * r.n + 8 * r.m;
        case HYD_REQ_LAPLACIAN: return 16 * r.n * r.m;
        case HYD_REQ_SPMV: return 28 * r.m + 8 * (r.n + 1) + 16 * r.n + 12 * r.n;
        default: return 0;
    }
}

static BatchInst spmv_inst(const hyd_request_t& r) {
    BatchInst I;
    memset(&I, 0, sizeof I);
    I.nrows = r.n;
    I.ncols = r.n;
    I.nnz = r.m;
    I.rows = static_cast<const int*>(r.in0);
    I.cols = static_cast<const int*>(r.in1);
    I.vals = static_cast<const double*>(r.in2);
    I.x = static_cast<const double*>(r.in3);
    I.y = static_cast<double*>(r.out0);
    I.row_ptr = static_cast<long long*>(r.out1);
    I.csr_cols = static_cast<int*>(r.out2);
    I.csr_vals = static_cast<double*>(r.out3);
    return I;
}

// Launches the mixed (dot / hist / laplacian) part of a batch on `s`.
// `host_tab` is pinned host memory kept alive until the stream passes this
// point; `key` names the slot's device scratch.
static int launch_mixed(const std::vector<const hyd_request_t*>& rq, const std::vector<int>& index, cudaStream_t s,
                        const std::string& key, void* host_tab, size_t host_tab_bytes, int* d_status) {
    if (rq.empty()) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    std::vector<MixReq> tab(rq.size());
    long long items = 0, words = 0;
    for (size_t i = 0; i < rq.size(); ++i) {
        const hyd_request_t& r = *rq[i];
        MixReq& M = tab[i];
        M.kind = r.kind;
        M.index = index[i];
        M.n = r.n;
        M.m = r.m;
        M.a = r.in0;
        M.b = r.in1;
        M.out = r.out0;
        M.item_base = items;
        M.scratch = words;
        if (r.kind == HYD_REQ_DOT) {
            M.nitems = r.n > 0 ? (r.n + kDotTile - 1) / kDotTile : 1;
            words += M.nitems;
        } else if (r.kind == HYD_REQ_HIST) {
            M.nitems = r.n > 0 ? (r.n + kHistTile - 1) / kHistTile : 1;
            words += M.nitems * r.m;
        } else {
            M.nitems = ((r.n + kLapTH - 1) / kLapTH) * ((r.m + kLapTW - 1) / kLapTW);
        }
        items += M.nitems;
    }
    const size_t tab_bytes = (tab.size() * sizeof(MixReq) + 255) & ~(size_t)255;
    const size_t done_bytes = (tab.size() * 4 + 255) & ~(size_t)255;
    const size_t scratch_bytes = (size_t)words * 8 + 256;
    void* buf = nullptr;
    HYD_TRY(device_buffer(d, key.c_str(), tab_bytes + done_bytes + 256 + scratch_bytes, &buf));
    unsigned char* b = static_cast<unsigned char*>(buf);
    MixReq* d_tab = reinterpret_cast<MixReq*>(b);
    unsigned* d_done = reinterpret_cast<unsigned*>(b + tab_bytes);
    unsigned* d_cursor = reinterpret_cast<unsigned*>(b + tab_bytes + done_bytes);
    unsigned long long* d_scratch = reinterpret_cast<unsigned long long*>(b + tab_bytes + done_bytes + 256);
    if (host_tab && host_tab_bytes >= tab.size() * sizeof(MixReq)) {
        memcpy(host_tab, tab.data(), tab.size() * sizeof(MixReq));
        HYD_CUDA_TRY(cudaMemcpyAsync(d_tab, host_tab, tab.size() * sizeof(MixReq), cudaMemcpyHostToDevice, s));
    } else {
        // pageable: the call returns once the table has been staged
        HYD_CUDA_TRY(cudaMemcpyAsync(d_tab, tab.data(), tab.size() * sizeof(MixReq), cudaMemcpyHostToDevice, s));
        HYD_CUDA_TRY(cudaStreamSynchronize(s));
    }
    HYD_CUDA_TRY(cudaMemsetAsync(d_done, 0, done_bytes + 256, s));
    HYD_TRY(configure_kernel((const void*)mixed_batch_kernel, d, false));
    long long grid = (long long)d->sm_count * 2;
    if (grid > items) grid = items;
    mixed_batch_kernel<<<(unsigned)grid, kMixThreads, kMixSmem, s>>>(d_tab, (int)tab.size(), items, d_cursor, d_done,
                                                                     d_scratch, d_status);
    return launch_check("mixed_batch");
}

// ---------------------------------------------------------------- server
struct TicketState {
    hyd_request_t req;
    long long bytes = 0;
    double t_arrive = 0.0, t_done = 0.0;
    int status = HYD_CUDA_OK;
    bool done = false;
};

struct Slot {
    int id = 0;
    cudaStream_t stream = nullptr;
    bool busy = false;
    std::vector<int64_t> tickets;
    long long bytes = 0;
    int* d_status = nullptr;      // device status per batch position
    int* h_status = nullptr;      // pinned copy read by the completion callback
    void* h_tab = nullptr;        // pinned staging for the mixed table
    void* h_spmv = nullptr;       // pinned staging for the SpMV tables
    size_t h_tab_bytes = 0, h_spmv_bytes = 0;
    int capacity = 0;
    struct Server* owner = nullptr;
};

struct Server {
    hyd_server_config_t cfg;
    std::mutex mu;
    std::condition_variable cv;  // dispatcher and waiters
    std::deque<TicketState> tickets;
    std::deque<int64_t> queue;
    std::vector<Slot*> slots;
    long long inflight = 0;
    hyd_server_stats_t stats;
    bool stopping = false;
    std::thread dispatcher;
    std::string error;  // message of the last failed batch (dispatcher thread)
    int device_id = 0;

    void run();
    int launch(Slot* sl, std::vector<int64_t>& batch);
};

static void CUDART_CB slot_done(void* p) {
    Slot* sl = static_cast<Slot*>(p);
    Server* sv = sl->owner;
    const double t = now_s();
    std::lock_guard<std::mutex> lock(sv->mu);
    for (size_t i = 0; i < sl->tickets.size(); ++i) {
        TicketState& T = sv->tickets[(size_t)sl->tickets[i]];
        T.status = sl->h_status[i];
        T.t_done = t;
        T.done = true;
        if (T.status == HYD_CUDA_OK) sv->stats.completed++;
        else sv->stats.failed++;
    }
    sv->inflight -= sl->bytes;
    sl->bytes = 0;
    sl->tickets.clear();
    sl->busy = false;
    sv->cv.notify_all();
}

int Server::launch(Slot* sl, std::vector<int64_t>& batch) {
    std::vector<const hyd_request_t*> mixed;
    std::vector<int> mixed_index;
    std::vector<BatchInst> spmv;
    for (size_t i = 0; i < batch.size(); ++i) {
        const hyd_request_t& r = tickets[(size_t)batch[i]].req;
        if (r.kind == HYD_REQ_SPMV) spmv.push_back(spmv_inst(r));
        else {
            mixed.push_back(&r);
            mixed_index.push_back((int)i);
        }
    }
    HYD_CUDA_TRY(cudaMemsetAsync(sl->d_status, 0, (size_t)batch.size() * 4, sl->stream));
    HYD_TRY(launch_mixed(mixed, mixed_index, sl->stream, "serve_mix_" + std::to_string(sl->id), sl->h_tab,
                         sl->h_tab_bytes, sl->d_status));
    if (!spmv.empty()) {
        const size_t need = batch_pipeline_table_bytes(spmv);
        if (need > sl->h_spmv_bytes) {
            // grow the pinned staging (the slot is idle on the host side here)
            if (sl->h_spmv) cudaFreeHost(sl->h_spmv);
            sl->h_spmv = nullptr;
            sl->h_spmv_bytes = 0;
            HYD_CUDA_TRY(cudaMallocHost(&sl->h_spmv, need * 2));
            sl->h_spmv_bytes = need * 2;
        }
        HYD_TRY(batch_pipeline(spmv, ("serve_spmv_" + std::to_string(sl->id)).c_str(), sl->stream, sl->h_spmv,
                               sl->h_spmv_bytes));
    }
    HYD_CUDA_TRY(cudaMemcpyAsync(sl->h_status, sl->d_status, (size_t)batch.size() * 4, cudaMemcpyDeviceToHost,
                                 sl->stream));
    HYD_CUDA_TRY(cudaLaunchHostFunc(sl->stream, slot_done, sl));
    return HYD_CUDA_OK;
}

void Server::run() {
    cudaSetDevice(device_id);
    std::unique_lock<std::mutex> lock(mu);
    for (;;) {
        Slot* free_slot = nullptr;
        for (Slot* s : slots)
            if (!s->busy) {
                free_slot = s;
                break;
            }
        if (stopping) {
            while (!queue.empty()) {
                TicketState& T = tickets[(size_t)queue.front()];
                T.status = HYD_CUDA_ERR_CANCELLED;
                T.t_done = now_s();
                T.done = true;
                stats.cancelled++;
                queue.pop_front();
            }
            bool any_busy = false;
            for (Slot* s : slots) any_busy |= s->busy;
            cv.notify_all();
            if (!any_busy) return;
            cv.wait(lock);
            continue;
        }
        if (queue.empty() || free_slot == nullptr) {
            cv.wait(lock);
            continue;
        }
        // admit FIFO while the working sets fit the budget and the batch has room
        std::vector<int64_t> batch;
        long long bytes = 0;
        while (!queue.empty() && (int)batch.size() < free_slot->capacity) {
            TicketState& T = tickets[(size_t)queue.front()];
            if (inflight + bytes + T.bytes > cfg.hbm_budget_bytes) break;
            if (!batch.empty() && bytes + T.bytes > cfg.max_batch_bytes) break;
            bytes += T.bytes;
            batch.push_back(queue.front());
            queue.pop_front();
        }
        if (batch.empty()) {  // waiting for memory to free up
            cv.wait(lock);
            continue;
        }
        inflight += bytes;
        if (inflight > stats.peak_inflight_bytes) stats.peak_inflight_bytes = inflight;
        free_slot->busy = true;
        free_slot->bytes = bytes;
        free_slot->tickets = batch;
        stats.launches++;
        lock.unlock();
        const int st = launch(free_slot, batch);
        lock.lock();
        if (st != HYD_CUDA_OK) {
            // nothing was enqueued behind a failed launch: fail the batch here
            error = last_error();
            cudaStreamSynchronize(free_slot->stream);
            for (int64_t t : batch) {
                TicketState& T = tickets[(size_t)t];
                T.status = st;
                T.t_done = now_s();
                T.done = true;
                stats.failed++;
            }
            inflight -= bytes;
            free_slot->bytes = 0;
            free_slot->tickets.clear();
            free_slot->busy = false;
            cv.notify_all();
        }
    }
}

static int submit_locked(Server* sv, const hyd_request_t* req, int64_t* ticket, double t_arrive) {
    TicketState T;
    T.req = *req;
    T.t_arrive = t_arrive;
    T.bytes = working_set(*req);
    const int v = validate(*req);
    sv->tickets.push_back(T);
    const int64_t id = (int64_t)sv->tickets.size() - 1;
    *ticket = id;
    sv->stats.submitted++;
    TicketState& S = sv->tickets.back();
    if (v != HYD_CUDA_OK || S.bytes > sv->cfg.hbm_budget_bytes || sv->stopping) {
        S.status = v != HYD_CUDA_OK ? v : (sv->stopping ? HYD_CUDA_ERR_CANCELLED : HYD_CUDA_ERR_BUDGET);
        S.t_done = t_arrive;
        S.done = true;
        if (S.status == HYD_CUDA_ERR_CANCELLED) sv->stats.cancelled++;
        else sv->stats.rejected++;
        return S.status;
    }
    sv->queue.push_back(id);
    sv->cv.notify_all();
    return HYD_CUDA_OK;
}

// Plain per-call execution of one request (what generated host code does
// without a server: one blocking call per invocation).
static int run_plain(const hyd_request_t& r, cudaStream_t s) {
    const int v = validate(r);
    if (v != HYD_CUDA_OK) return set_error(v, "request of kind %d is invalid", r.kind);
    switch (r.kind) {
        case HYD_REQ_DOT:
            HYD_TRY(hyd_cuda_dot_f64((const double*)r.in0, (const double*)r.in1, r.n, (double*)r.out0, s));
            break;
        case HYD_REQ_HIST:
            HYD_CUDA_TRY(cudaMemsetAsync(r.out0, 0, (size_t)r.m * 8, s));
            HYD_TRY(hyd_cuda_weighted_histogram_i64((const int64_t*)r.in0, r.n, r.m, (int64_t*)r.out0,
                                                    HYD_SCATTER_AUTO, s));
            break;
        case HYD_REQ_LAPLACIAN:
            HYD_TRY(hyd_cuda_stencil2d_f64(HYD_STENCIL_LAPLACIAN, (const double*)r.in0, (double*)r.out0, r.n, r.m, s));
            break;
        case HYD_REQ_SPMV: {
            std::vector<BatchInst> one{spmv_inst(r)};
            HYD_TRY(batch_pipeline(one, "plain_spmv", s, nullptr, 0));
            break;
        }
    }
    return hyd_cuda_check(s);
}

}  // namespace hyd

using namespace hyd;

struct hyd_server {
    Server impl;
};

extern "C" int hyd_cuda_server_create(const hyd_server_config_t* cfg, hyd_server_t** out) {
    HYD_CHECK_ARG(out != nullptr, "server_create: null out");
    Device* d = nullptr;
    HYD_TRY(device(&d));
    hyd_server_t* h = new hyd_server_t();
    Server& sv = h->impl;
    memset(&sv.stats, 0, sizeof sv.stats);
    hyd_server_config_t c;
    memset(&c, 0, sizeof c);
    if (cfg) c = *cfg;
    if (c.hbm_budget_bytes <= 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        c.hbm_budget_bytes = (int64_t)(fr / 4);
    }
    if (c.streams <= 0) c.streams = 4;
    if (c.streams > 16) c.streams = 16;
    if (c.max_batch <= 0) c.max_batch = 256;
    if (c.max_batch_bytes <= 0) c.max_batch_bytes = c.hbm_budget_bytes / c.streams;
    sv.cfg = c;
    sv.device_id = d->id;
    for (int i = 0; i < c.streams; ++i) {
        Slot* s = new Slot();
        s->id = i;
        s->owner = &sv;
        s->capacity = c.max_batch;
        int e = HYD_CUDA_OK;
        if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaMalloc(&s->d_status, (size_t)c.max_batch * 4) != cudaSuccess ||
            cudaMallocHost(&s->h_status, (size_t)c.max_batch * 4) != cudaSuccess ||
            cudaMallocHost(&s->h_tab, (size_t)c.max_batch * sizeof(MixReq)) != cudaSuccess)
            e = HYD_CUDA_ERR_NOMEM;
        s->h_tab_bytes = (size_t)c.max_batch * sizeof(MixReq);
        sv.slots.push_back(s);
        if (e != HYD_CUDA_OK) {
            hyd_cuda_server_destroy(h);
            return set_error(e, "server_create: slot allocation failed");
        }
    }
    sv.dispatcher = std::thread([&sv] { sv.run(); });
    *out = h;
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_server_submit(hyd_server_t* srv, const hyd_request_t* req, int64_t* ticket) {
    HYD_CHECK_ARG(srv && req && ticket, "server_submit: null argument");
    std::lock_guard<std::mutex> lock(srv->impl.mu);
    return submit_locked(&srv->impl, req, ticket, now_s());
}

extern "C" int hyd_cuda_server_wait(hyd_server_t* srv, int64_t ticket, int* status, double* latency_s) {
    HYD_CHECK_ARG(srv != nullptr, "server_wait: null server");
    Server& sv = srv->impl;
    std::unique_lock<std::mutex> lock(sv.mu);
    HYD_CHECK_ARG(ticket >= 0 && ticket < (int64_t)sv.tickets.size(), "server_wait: unknown ticket");
    sv.cv.wait(lock, [&] { return sv.tickets[(size_t)ticket].done; });
    const TicketState& T = sv.tickets[(size_t)ticket];
    if (status) *status = T.status;
    if (latency_s) *latency_s = T.t_done - T.t_arrive;
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_server_stats(hyd_server_t* srv, hyd_server_stats_t* out) {
    HYD_CHECK_ARG(srv && out, "server_stats: null argument");
    std::lock_guard<std::mutex> lock(srv->impl.mu);
    *out = srv->impl.stats;
    out->inflight_bytes = srv->impl.inflight;
    out->queued = (int64_t)srv->impl.queue.size();
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_server_shutdown(hyd_server_t* srv) {
    HYD_CHECK_ARG(srv != nullptr, "server_shutdown: null server");
    Server& sv = srv->impl;
    {
        std::lock_guard<std::mutex> lock(sv.mu);
        sv.stopping = true;
        sv.cv.notify_all();
    }
    if (sv.dispatcher.joinable()) sv.dispatcher.join();
    return HYD_CUDA_OK;
}

extern "C" const char* hyd_cuda_server_error(hyd_server_t* srv) {
    if (!srv) return "";
    std::lock_guard<std::mutex> lock(srv->impl.mu);
    static thread_local std::string copy;
    copy = srv->impl.error;
    return copy.c_str();
}

extern "C" int hyd_cuda_server_destroy(hyd_server_t* srv) {
    if (!srv) return HYD_CUDA_OK;
    Server& sv = srv->impl;
    hyd_cuda_server_shutdown(srv);
    for (Slot* s : sv.slots) {
        if (s->stream) {
            cudaStreamSynchronize(s->stream);
            cudaStreamDestroy(s->stream);
        }
        if (s->d_status) cudaFree(s->d_status);
        if (s->h_status) cudaFreeHost(s->h_status);
        if (s->h_tab) cudaFreeHost(s->h_tab);
        if (s->h_spmv) cudaFreeHost(s->h_spmv);
        delete s;
    }
    delete srv;
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_request_run(const hyd_request_t* req, void* stream) {
    HYD_CHECK_ARG(req != nullptr, "request_run: null request");
    return run_plain(*req, as_stream(stream));
}

static void wait_until(double t) {
    for (;;) {
        const double now = now_s();
        if (now >= t) return;
        if (t - now > 2e-3) std::this_thread::sleep_for(std::chrono::microseconds(500));
    }
}

extern "C" int hyd_cuda_serve_trace(hyd_server_t* srv, const hyd_request_t* reqs, const double* arrival_s, int64_t n,
                                    double* latency_s, int* status, double* elapsed_s) {
    HYD_CHECK_ARG(srv && (n == 0 || (reqs && arrival_s && latency_s && status)), "serve_trace: null argument");
    Server& sv = srv->impl;
    std::vector<int64_t> ids((size_t)n);
    const double t0 = now_s();
    for (int64_t i = 0; i < n; ++i) {
        wait_until(t0 + arrival_s[i]);
        std::lock_guard<std::mutex> lock(sv.mu);
        submit_locked(&sv, &reqs[i], &ids[(size_t)i], t0 + arrival_s[i]);
    }
    double last = t0;
    for (int64_t i = 0; i < n; ++i) {
        double lat = 0.0;
        hyd_cuda_server_wait(srv, ids[(size_t)i], &status[i], &lat);
        latency_s[i] = lat;
        std::lock_guard<std::mutex> lock(sv.mu);
        last = std::max(last, sv.tickets[(size_t)ids[(size_t)i]].t_done);
    }
    if (elapsed_s) *elapsed_s = last - t0;
    return HYD_CUDA_OK;
}

extern "C" int hyd_cuda_plain_trace(const hyd_request_t* reqs, const double* arrival_s, int64_t n, double* latency_s,
                                    int* status, double* elapsed_s, void* stream) {
    HYD_CHECK_ARG(n == 0 || (reqs && arrival_s && latency_s && status), "plain_trace: null argument");
    cudaStream_t s = as_stream(stream);
    const double t0 = now_s();
    double last = t0;
    for (int64_t i = 0; i < n; ++i) {
        wait_until(t0 + arrival_s[i]);
        status[i] = run_plain(reqs[i], s);
        last = now_s();
        latency_s[i] = last - (t0 + arrival_s[i]);
    }
    if (elapsed_s) *elapsed_s = last - t0;
    return HYD_CUDA_OK;
}
