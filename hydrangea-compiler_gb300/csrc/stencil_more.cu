// stencil_more.cu -- the other iterate loops of the stencil family:
//  * jacobi_1d: the 1-D clamp 3-point mean (examples/jacobi_1d.hyd:4),
//    out[i] = (in[i-1] + in[i] + in[i+1]) / 3.0 with clamped neighbours;
//  * gray_scott: one two-field reaction-diffusion step with periodic
//    neighbours (demo/gray_scott/gray_scott.hyd:47-73), and the demo's
//    zero-argument export hyd_export_gray_scott (its 5000 steps from the
//    program's initial fields).
// Every expression is evaluated in the program's order with IEEE
// round-to-nearest operations (no contraction), so results are bit-identical
// to the C backend.  `x - 4.0*y` is one fma: 4y is exact, so RN(x - 4y) is the
// C result.  Sums of two non-negative operands may run on the integer pipe
// (dadd_pos, exact).  Iterations are captured once into a CUDA graph per
// (shape, buffers, count, stream) and replayed.
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "fp64_emu.cuh"
#include "hyd_common.cuh"

namespace hyd {

__global__ void jacobi1d_kernel(const double* __restrict__ in, double* __restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t l = i > 0 ? i - 1 : 0, r = i + 1 < n ? i + 1 : n - 1;
        const double s = dadd_pos(dadd_pos(in[l], in[i]), in[r]);
        out[i] = ddiv_small_rn<3>(s);  // = __ddiv_rn(s, 3.0), bit for bit
    }
}

struct GsParams {
    double du, dv, feed, kill, dt;
    double feed_kill;  // feed + kill, rounded once on the host: the same double as the program's per-point sum
};

// kUnitDt: dt == 1.0, so dt * t == t exactly and the multiplication is left
// out.  Of each Laplacian's three neighbour additions the first two run on the
// integer pipe (exact; the FP64 unit for negative operands).  GB300's FP64
// unit (1.9 operations per clock per SM) bounds this kernel.
template <bool kUnitDt>
__global__ void __launch_bounds__(256) gray_scott_kernel(const double* __restrict__ u, const double* __restrict__ v,
                                                         double* __restrict__ un, double* __restrict__ vn,
                                                         int64_t h, int64_t w, GsParams p) {
    const int64_t j = (int64_t)blockIdx.x * 32 + (threadIdx.x & 31);
    const int64_t i = (int64_t)blockIdx.y * 8 + (threadIdx.x >> 5);
    if (i >= h || j >= w) return;
    // imod (i - 1 + h) h and imod (i + 1) h of the program
    const int64_t im = i > 0 ? i - 1 : h - 1, ip = i + 1 < h ? i + 1 : 0;
    const int64_t jm = j > 0 ? j - 1 : w - 1, jp = j + 1 < w ? j + 1 : 0;
    const double uij = u[i * w + j], vij = v[i * w + j];
    double lu = __dadd_rn(dadd_pos(dadd_pos(u[im * w + j], u[ip * w + j]), u[i * w + jm]), u[i * w + jp]);
    lu = __fma_rn(-4.0, uij, lu);
    double lv = __dadd_rn(dadd_pos(dadd_pos(v[im * w + j], v[ip * w + j]), v[i * w + jm]), v[i * w + jp]);
    lv = __fma_rn(-4.0, vij, lv);
    const double uvv = __dmul_rn(__dmul_rn(uij, vij), vij);
    double tu = __dsub_rn(__dmul_rn(p.du, lu), uvv);
    tu = __dadd_rn(tu, __dmul_rn(p.feed, __dsub_rn(1.0, uij)));
    un[i * w + j] = __dadd_rn(uij, kUnitDt ? tu : __dmul_rn(p.dt, tu));
    double tv = __dadd_rn(__dmul_rn(p.dv, lv), uvv);
    tv = __dsub_rn(tv, __dmul_rn(p.feed_kill, vij));
    vn[i * w + j] = __dadd_rn(vij, kUnitDt ? tv : __dmul_rn(p.dt, tv));
}

// The demo's initial fields (gray_scott.hyd:28-39): U = 1; V = 0.5 inside the
// centre disk of radius 20 and at sparse seed points, else 0.
__global__ void gray_scott_init_kernel(double* __restrict__ u, double* __restrict__ v, int64_t h, int64_t w) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < h * w; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k / w, j = k % w;
        const int64_t di = i - h / 2, dj = j - w / 2;
        u[k] = 1.0;
        v[k] = (di * di + dj * dj < 20 * 20) ? 0.5 : ((i * 251 + j * 127) % 100 < 2 ? 0.5 : 0.0);
    }
}

static int launch_jacobi1d(const double* in, double* out, int64_t n, const Device* d, cudaStream_t s) {
    const int64_t want = (n + 255) / 256;
    const int64_t cap = (int64_t)d->sm_count * 8;
    jacobi1d_kernel<<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(in, out, n);
    return launch_check("jacobi1d_f64");
}

static int launch_gray_scott(const double* u, const double* v, double* un, double* vn, int64_t h, int64_t w,
                             const GsParams& p, cudaStream_t s) {
    dim3 grid((unsigned)((w + 31) / 32), (unsigned)((h + 7) / 8));
    if (p.dt == 1.0) gray_scott_kernel<true><<<grid, 256, 0, s>>>(u, v, un, vn, h, w, p);
    else gray_scott_kernel<false><<<grid, 256, 0, s>>>(u, v, un, vn, h, w, p);
    return launch_check("gray_scott_f64");
}

// Captured step sequences, keyed by (kind, shape, parameters, buffers, count, stream).
struct MoreKey {
    int kind;
    int64_t h, w, iters;
    const void *b0, *b1, *b2, *b3;
    double p[5];
    cudaStream_t stream;
    bool operator<(const MoreKey& o) const {
        return std::tie(kind, h, w, iters, b0, b1, b2, b3, p[0], p[1], p[2], p[3], p[4], stream) <
               std::tie(o.kind, o.h, o.w, o.iters, o.b0, o.b1, o.b2, o.b3, o.p[0], o.p[1], o.p[2], o.p[3], o.p[4],
                        o.stream);
    }
};
static std::mutex g_more_mu;
static std::map<MoreKey, cudaGraphExec_t> g_more_graphs;

void release_more_graphs() {
    std::lock_guard<std::mutex> lock(g_more_mu);
    for (auto& kv : g_more_graphs) cudaGraphExecDestroy(kv.second);
    g_more_graphs.clear();
}

// Runs `step(t)` for t < iters on `st`: eagerly on the legacy stream or for
// fewer than 4 steps, otherwise as a cached captured graph.
template <class Step>
static int run_steps(const MoreKey& key, cudaStream_t st, int64_t iters, Step step) {
    if (st == nullptr || iters < 4) {
        for (int64_t t = 0; t < iters; ++t) HYD_TRY(step(t));
        return HYD_CUDA_OK;
    }
    cudaGraphExec_t exec = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_more_mu);
        auto it = g_more_graphs.find(key);
        if (it != g_more_graphs.end()) exec = it->second;
    }
    if (!exec) {
        cudaGraph_t graph = nullptr;
        HYD_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int status = HYD_CUDA_OK;
        for (int64_t t = 0; t < iters && status == HYD_CUDA_OK; ++t) status = step(t);
        cudaError_t ce = cudaStreamEndCapture(st, &graph);
        if (status != HYD_CUDA_OK) {
            if (graph) cudaGraphDestroy(graph);
            return status;
        }
        HYD_CUDA_TRY(ce);
        cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        HYD_CUDA_TRY(ie);
        std::lock_guard<std::mutex> lock(g_more_mu);
        if (g_more_graphs.size() >= 64) {  // bounded cache: drop everything when full
            for (auto& kv : g_more_graphs) cudaGraphExecDestroy(kv.second);
            g_more_graphs.clear();
        }
        g_more_graphs[key] = exec;
    }
    HYD_CUDA_TRY(cudaGraphLaunch(exec, st));
    return HYD_CUDA_OK;
}

static GsParams gs_params(const hyd_gray_scott_t* p) {
    GsParams g = p ? GsParams{p->du, p->dv, p->feed, p->kill, p->dt, 0.0}
                   : GsParams{0.21, 0.105, 0.0545, 0.0620, 1.0, 0.0};  // gray_scott.hyd:19-25
    volatile double f = g.feed, k = g.kill;  // one IEEE double addition, as the program's per-point sum
    g.feed_kill = f + k;
    return g;
}

}  // namespace hyd

using namespace hyd;

extern "C" {

int hyd_cuda_jacobi1d_f64(const double* in, double* out, int64_t n, void* stream) {
    HYD_CHECK_ARG(n >= 0 && (n == 0 || (in && out && in != out)), "jacobi1d: bad arguments");
    if (n == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    return launch_jacobi1d(in, out, n, d, as_stream(stream));
}

int hyd_cuda_iterate_jacobi1d_f64(double* buf0, double* buf1, int64_t n, int64_t iters, int* final_buf,
                                  void* stream) {
    HYD_CHECK_ARG(n >= 0 && iters >= 0 && final_buf != nullptr, "iterate_jacobi1d: bad arguments");
    HYD_CHECK_ARG(n == 0 || (buf0 && buf1 && buf0 != buf1), "iterate_jacobi1d: need two distinct buffers");
    *final_buf = (int)(iters & 1);
    if (n == 0 || iters == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    cudaStream_t st = as_stream(stream);
    double* b[2] = {buf0, buf1};
    MoreKey key{1, 1, n, iters, buf0, buf1, nullptr, nullptr, {0, 0, 0, 0, 0}, st};
    return run_steps(key, st, iters, [&](int64_t t) { return launch_jacobi1d(b[t & 1], b[(t + 1) & 1], n, d, st); });
}

int hyd_cuda_gray_scott_step_f64(const double* u, const double* v, double* u_out, double* v_out, int64_t h,
                                 int64_t w, const hyd_gray_scott_t* params, void* stream) {
    HYD_CHECK_ARG(h >= 0 && w >= 0, "gray_scott_step: negative shape");
    HYD_CHECK_ARG(h * w == 0 || (u && v && u_out && v_out), "gray_scott_step: null buffer");
    HYD_CHECK_ARG(u != u_out && v != v_out && u_out != v_out, "gray_scott_step: outputs must be distinct buffers");
    if (h == 0 || w == 0) return HYD_CUDA_OK;
    return launch_gray_scott(u, v, u_out, v_out, h, w, gs_params(params), as_stream(stream));
}

int hyd_cuda_iterate_gray_scott_f64(double* u0, double* v0, double* u1, double* v1, int64_t h, int64_t w,
                                    const hyd_gray_scott_t* params, int64_t steps, int* final_buf, void* stream) {
    HYD_CHECK_ARG(h >= 0 && w >= 0 && steps >= 0 && final_buf != nullptr, "iterate_gray_scott: bad arguments");
    HYD_CHECK_ARG(h * w == 0 || (u0 && v0 && u1 && v1), "iterate_gray_scott: null buffer");
    HYD_CHECK_ARG(u0 != u1 && v0 != v1 && u0 != v0 && u1 != v1 && u0 != v1 && u1 != v0,
                  "iterate_gray_scott: four distinct buffers");
    *final_buf = (int)(steps & 1);
    if (h == 0 || w == 0 || steps == 0) return HYD_CUDA_OK;
    Device* d = nullptr;
    HYD_TRY(device(&d));
    cudaStream_t st = as_stream(stream);
    const GsParams p = gs_params(params);
    double* us[2] = {u0, u1};
    double* vs[2] = {v0, v1};
    MoreKey key{2, h, w, steps, u0, u1, v0, v1, {p.du, p.dv, p.feed, p.kill, p.dt}, st};
    return run_steps(key, st, steps, [&](int64_t t) {
        return launch_gray_scott(us[t & 1], vs[t & 1], us[(t + 1) & 1], vs[(t + 1) & 1], h, w, p, st);
    });
}

// The demo's procedure (gray_scott.hyd:80, called by demo/gray_scott/main.cpp:85):
// V after 5000 steps on the 256 x 256 grid, computed into a fresh host array.
// Failures keep the reference's behaviour (stderr, exit 1).
static hyd_array_t* gray_scott_compute(void) {
    const int64_t h = 256, w = 256, steps = 5000;
    hyd_tuple_t shape;
    shape.ndims = 2;
    shape.elems[0] = h;
    shape.elems[1] = w;
    hyd_array_t* out = hyd_cuda_array_alloc(shape, sizeof(double));
    if (!out) {
        fprintf(stderr, "hydrangea(cuda): hyd_export_gray_scott: host allocation failed\n");
        exit(1);
    }
    Device* d = nullptr;
    double* buf = nullptr;
    int st = device(&d);
    if (st == HYD_CUDA_OK && cudaMalloc(&buf, (size_t)(4 * h * w) * sizeof(double)) != cudaSuccess)
        st = set_error(HYD_CUDA_ERR_NOMEM, "gray_scott: device allocation failed");
    cudaStream_t s = nullptr;
    if (st == HYD_CUDA_OK && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
        st = set_error(HYD_CUDA_ERR_CUDA, "gray_scott: stream creation failed");
    int which = 0;
    if (st == HYD_CUDA_OK) {
        gray_scott_init_kernel<<<(unsigned)(d->sm_count * 4), 256, 0, s>>>(buf, buf + h * w, h, w);
        st = launch_check("gray_scott_init");
    }
    if (st == HYD_CUDA_OK)
        st = hyd_cuda_iterate_gray_scott_f64(buf, buf + h * w, buf + 2 * h * w, buf + 3 * h * w, h, w, nullptr,
                                             steps, &which, s);
    if (st == HYD_CUDA_OK &&
        cudaMemcpyAsync(out->data, buf + (which ? 3 : 1) * h * w, (size_t)(h * w) * sizeof(double),
                        cudaMemcpyDeviceToHost, s) != cudaSuccess)
        st = set_error(HYD_CUDA_ERR_CUDA, "gray_scott: copy failed");
    if (st == HYD_CUDA_OK && cudaStreamSynchronize(s) != cudaSuccess)
        st = set_error(HYD_CUDA_ERR_CUDA, "gray_scott: synchronize failed");
    if (st == HYD_CUDA_OK) st = hyd_cuda_check(s);
    if (s) {
        std::lock_guard<std::mutex> lock(g_more_mu);  // the cached graph names this stream
        for (auto it = g_more_graphs.begin(); it != g_more_graphs.end();) {
            if (it->first.stream == s) {
                cudaGraphExecDestroy(it->second);
                it = g_more_graphs.erase(it);
            } else {
                ++it;
            }
        }
    }
    if (s) cudaStreamDestroy(s);
    if (buf) cudaFree(buf);
    if (st != HYD_CUDA_OK) {
        fprintf(stderr, "hydrangea(cuda): hyd_export_gray_scott failed: %s (%s)\n", hyd_cuda_status_string(st),
                last_error());
        exit(1);
    }
    return out;
}

// Like every zero-argument array procedure of the reference's C backend
// (CodegenC.hs:690-707, :812-833), the export is memoised: the first call
// computes the array and keeps one reference to it; every call returns a view,
// a new header over the same storage with its reference count raised, which
// the caller frees with hyd_array_free (runtime/hydrangea_runtime.h:319-343).
// hyd_cuda_cleanup drops the runtime's own reference.
static std::mutex g_gs_memo_mu;
static hyd_array_t* g_gs_memo = nullptr;

hyd_array_t* hyd_export_gray_scott(void) {
    std::lock_guard<std::mutex> lock(g_gs_memo_mu);
    if (!g_gs_memo) g_gs_memo = gray_scott_compute();
    hyd_array_t* view = (hyd_array_t*)malloc(sizeof(hyd_array_t));
    if (!view) {
        fprintf(stderr, "hydrangea(cuda): hyd_export_gray_scott: host allocation failed\n");
        exit(1);
    }
    *view = *g_gs_memo;
    view->data = g_gs_memo->storage->data;
    g_gs_memo->storage->refcount += 1;
    return view;
}

}  // extern "C"

namespace hyd {

// What hyd_array_free does to the runtime's reference of each memoised export.
void release_export_memos() {
    std::lock_guard<std::mutex> lock(g_gs_memo_mu);
    if (!g_gs_memo) return;
    hyd_array_storage_t* st = g_gs_memo->storage;
    st->refcount -= 1;
    if (st->refcount == 0) {
        free(st->data);
        free(st);
    }
    free(g_gs_memo);
    g_gs_memo = nullptr;
}

}  // namespace hyd
