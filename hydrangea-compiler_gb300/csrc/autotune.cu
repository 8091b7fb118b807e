// autotune.cu -- the project's autotuner: per (kernel, shape class) choice of
// tile shape / privatisation strategy, measured on the device and cached on
// disk.
//
// The reference fixes its tiling at compile time (the polyhedral scheduler's
// 32 x 32 tiles, Polyhedral.hs:196-210) and its scatter strategy by a static
// cap (Parallelize.hs:492).  Here every tunable kernel has a list of
// candidates that all give bit-identical results; tuning times each candidate
// on scratch inputs of the requested shape with CUDA events (median of reps)
// and records the fastest.  AUTO launches consult the table.
//
// Table: key = (device name, kernel, shape class) -> (choice, microseconds).
// Persisted as tab-separated lines "device kernel class choice us" appended to
// $HYD_CUDA_TUNE_CACHE (default $HOME/.cache/hydrangea_cuda_tune.tsv); on first
// use the file is read and the last line for a key wins.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "hyd_common.cuh"

namespace hyd {

struct TuneVal {
    int choice;
    double us;
};

static std::mutex g_tune_mu;
static std::map<std::string, TuneVal> g_tune;
static bool g_tune_loaded = false;
static std::string g_tune_path;

static std::string key_of(const std::string& dev, const std::string& kernel, const std::string& klass) {
    return dev + "\t" + kernel + "\t" + klass;
}

static std::string default_path() {
    const char* p = getenv("HYD_CUDA_TUNE_CACHE");
    if (p && *p) return p;
    const char* home = getenv("HOME");
    return std::string(home && *home ? home : ".") + "/.cache/hydrangea_cuda_tune.tsv";
}

static void load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    if (g_tune_path.empty()) g_tune_path = default_path();
    FILE* f = fopen(g_tune_path.c_str(), "r");
    if (!f) return;
    char line[1024];
    while (fgets(line, sizeof line, f)) {
        std::vector<std::string> parts;
        std::string cur;
        for (const char* c = line; *c && *c != '\n'; ++c) {
            if (*c == '\t') {
                parts.push_back(cur);
                cur.clear();
            } else {
                cur.push_back(*c);
            }
        }
        parts.push_back(cur);
        if (parts.size() != 5) continue;
        g_tune[key_of(parts[0], parts[1], parts[2])] = TuneVal{atoi(parts[3].c_str()), atof(parts[4].c_str())};
    }
    fclose(f);
}

static void record(const std::string& dev, const std::string& kernel, const std::string& klass, int choice,
                   double us) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    load_locked();
    g_tune[key_of(dev, kernel, klass)] = TuneVal{choice, us};
    FILE* f = fopen(g_tune_path.c_str(), "a");
    if (!f) {
        // create the parent directories (mkdir -p), then retry once
        const size_t slash = g_tune_path.find_last_of('/');
        if (slash != std::string::npos && slash > 0) {
            const std::string dir = g_tune_path.substr(0, slash);
            for (size_t i = 1; i <= dir.size(); ++i)
                if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);
        }
        f = fopen(g_tune_path.c_str(), "a");
        if (!f) return;  // the in-memory table still holds the choice
    }
    fprintf(f, "%s\t%s\t%s\t%d\t%.3f\n", dev.c_str(), kernel.c_str(), klass.c_str(), choice, us);
    fclose(f);
}

static int query(const std::string& dev, const std::string& kernel, const std::string& klass) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    load_locked();
    auto it = g_tune.find(key_of(dev, kernel, klass));
    return it == g_tune.end() ? -1 : it->second.choice;
}

static std::string current_device_name() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return "none";
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        return "none";
    }
    std::string name = prop.name;
    for (char& c : name)
        if (c == '\t' || c == '\n') c = ' ';
    return name + "/sm" + std::to_string(prop.major) + std::to_string(prop.minor) + "x" +
           std::to_string(prop.multiProcessorCount);
}

static std::string cached_device_name() {
    static std::mutex mu;
    static std::vector<std::string> names;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return "none";
    }
    std::lock_guard<std::mutex> lock(mu);
    if ((int)names.size() <= dev) names.resize(dev + 1);
    if (names[dev].empty()) names[dev] = current_device_name();
    return names[dev];
}

static int log2c(long long v) {
    int s = 0;
    while ((1LL << s) < v) ++s;
    return s;
}

std::string stencil_class(int kind, int64_t h, int64_t w) {
    return "k" + std::to_string(kind) + "_h" + std::to_string(log2c(h)) + "_w" + std::to_string(log2c(w));
}
std::string hist_class(int64_t bins) { return "b" + std::to_string(log2c(bins)); }

int tune_lookup_stencil(int kind, int64_t h, int64_t w) {
    return query(cached_device_name(), "stencil2d", stencil_class(kind, h, w));
}
int tune_lookup_hist(int64_t bins) { return query(cached_device_name(), "weighted_histogram", hist_class(bins)); }

template <class F>
static int time_us(F launch, int reps, cudaStream_t s, double* out_us) {
    cudaEvent_t e0, e1;
    HYD_CUDA_TRY(cudaEventCreate(&e0));
    HYD_CUDA_TRY(cudaEventCreate(&e1));
    std::vector<float> ts;
    int st = launch();  // warm-up
    for (int r = 0; r < reps && st == HYD_CUDA_OK; ++r) {
        cudaEventRecord(e0, s);
        st = launch();
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ts.push_back(ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != HYD_CUDA_OK) return st;
    std::sort(ts.begin(), ts.end());
    *out_us = ts.empty() ? 0.0 : 1000.0 * ts[ts.size() / 2];
    return HYD_CUDA_OK;
}

}  // namespace hyd

using namespace hyd;

extern "C" int hyd_cuda_stencil2d_f64_variant(int kind, const double* in, double* out, int64_t h, int64_t w,
                                              int variant, void* stream);

extern "C" {

const char* hyd_cuda_tune_cache_path(void) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (g_tune_path.empty()) g_tune_path = default_path();
    return g_tune_path.c_str();
}

int hyd_cuda_tune_set_cache_path(const char* path) {
    HYD_CHECK_ARG(path != nullptr && *path, "tune_set_cache_path: empty path");
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune.clear();
    g_tune_loaded = false;
    g_tune_path = path;
    load_locked();
    return HYD_CUDA_OK;
}

int hyd_cuda_tune_record(const char* device, const char* kernel, const char* klass, int choice, double us) {
    HYD_CHECK_ARG(kernel && klass && choice >= 0, "tune_record: bad arguments");
    record(device ? device : cached_device_name(), kernel, klass, choice, us);
    return HYD_CUDA_OK;
}

int hyd_cuda_tune_query(const char* device, const char* kernel, const char* klass) {
    if (!kernel || !klass) return -1;
    return query(device ? device : cached_device_name(), kernel, klass);
}

int hyd_cuda_autotune_stencil2d(int kind, int64_t h, int64_t w, int reps, int* best, double* times_us) {
    HYD_CHECK_ARG(kind >= 0 && kind <= 3 && h >= 1 && w >= 2 && reps >= 1, "autotune_stencil2d: bad arguments");
    HYD_CHECK_ARG(best != nullptr, "autotune_stencil2d: null best");
    double *a = nullptr, *b = nullptr;
    HYD_CUDA_TRY(cudaMalloc(&a, (size_t)h * w * 8));
    cudaError_t e = cudaMalloc(&b, (size_t)h * w * 8);
    if (e != cudaSuccess) {
        cudaFree(a);
        return set_error(HYD_CUDA_ERR_NOMEM, "autotune_stencil2d: scratch allocation failed");
    }
    cudaStream_t s = nullptr;
    int st = hyd_cuda_fill_uniform_f64(a, h * w, 99, 0.0, 1.0, s);
    const int nvar = 21;  // 7 shapes x 3 integer-pipe levels
    double best_us = 1e300;
    int best_v = -1;
    for (int v = 0; v < nvar && st == HYD_CUDA_OK; ++v) {
        double us = 0.0;
        st = time_us([&] { return hyd_cuda_stencil2d_f64_variant(kind, a, b, h, w, v, s); }, reps, s, &us);
        if (times_us) times_us[v] = us;
        if (st == HYD_CUDA_OK && us < best_us) {
            best_us = us;
            best_v = v;
        }
    }
    cudaFree(a);
    cudaFree(b);
    if (st != HYD_CUDA_OK) return st;
    *best = best_v;
    record(cached_device_name(), "stencil2d", stencil_class(kind, h, w), best_v, best_us);
    return HYD_CUDA_OK;
}

int hyd_cuda_autotune_histogram(int64_t n, int64_t bins, int reps, int* best, double* times_us) {
    HYD_CHECK_ARG(n >= 1 && bins >= 1 && reps >= 1 && best != nullptr, "autotune_histogram: bad arguments");
    int64_t *data = nullptr, *hist = nullptr;
    HYD_CUDA_TRY(cudaMalloc(&data, (size_t)n * 8));
    cudaError_t e = cudaMalloc(&hist, (size_t)bins * 8);
    if (e != cudaSuccess) {
        cudaFree(data);
        return set_error(HYD_CUDA_ERR_NOMEM, "autotune_histogram: scratch allocation failed");
    }
    cudaStream_t s = nullptr;
    int st = hyd_cuda_fill_uniform_i64(data, n, 2, 1LL << 20, s);
    double best_us = 1e300;
    int best_v = -1;
    for (int v = HYD_SCATTER_SMEM_WARP; v <= HYD_SCATTER_PARTITION && st == HYD_CUDA_OK; ++v) {
        double us = 0.0;
        const int r = time_us([&] { return hyd_cuda_weighted_histogram_i64(data, n, bins, hist, v, s); }, reps, s, &us);
        if (times_us) times_us[v] = r == HYD_CUDA_OK ? us : -1.0;
        if (r == HYD_CUDA_OK && us < best_us) {
            best_us = us;
            best_v = v;
        }
        if (r != HYD_CUDA_OK && r != HYD_CUDA_ERR_UNSUPPORTED) st = r;
    }
    cudaFree(data);
    cudaFree(hist);
    if (st != HYD_CUDA_OK) return st;
    if (best_v < 0) return set_error(HYD_CUDA_ERR_UNSUPPORTED, "autotune_histogram: no strategy ran");
    *best = best_v;
    record(cached_device_name(), "weighted_histogram", hist_class(bins), best_v, best_us);
    return HYD_CUDA_OK;
}

}  // extern "C"
