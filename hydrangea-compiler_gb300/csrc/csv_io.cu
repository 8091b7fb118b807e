// csv_io.cu -- the host I/O path: CSV files to arrays (host or device) and back.
//
// The reference's generated code reads its inputs with hyd_read_array_csv /
// hyd_read_float_array_csv (runtime/hydrangea_runtime.h:549-592) and writes
// results with hyd_write_array_csv[_float] (runtime/hyd_write_csv.c).  Their
// grammar, reproduced here exactly:
//   * element i > 0 is preceded by a skip over ',' ' ' '\n' '\r'; reaching the
//     end of the file there is "too few values";
//   * fscanf("%lld" / "%lf") then skips white space and converts the longest
//     number prefix; no conversion is "parse error at element i";
//   * exactly `size` elements are read; the rest of the file is ignored;
//   * output rows are "%lld" / "%.17g" values joined by ',' and ended by '\n'
//     (one row per row of a 2-D array, else one row).
// Reading runs on all host threads: the file is split at token starts (a
// token is a maximal run of characters that are neither ',' nor white
// space), each thread converts its tokens and checks the separator run before
// each one, and the slices are joined in order.  Tokens of the usual forms
// ([+-]digits within int64; decimal floats with an optional exponent,
// converted by strtod, which rounds as the C library's scanf does) take that
// path; a file whose first `size` tokens hold anything else (hexadecimal or
// infinite values, trailing characters, out-of-range integers) is read again
// by a sequential pass that hands each token to sscanf -- the C library's own
// scanf engine -- so every case, errors included, behaves as fscanf does.
// The device forms parse into pinned memory and copy to or from the device.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "hyd_common.cuh"

namespace hyd {

namespace {

inline bool is_skip(unsigned char c) { return c == ',' || c == ' ' || c == '\n' || c == '\r'; }
inline bool is_ws(unsigned char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }
inline bool is_sep(unsigned char c) { return c == ',' || is_ws(c); }

struct CsvError {
    int kind = 0;  // 0 none, 1 too few values, 2 parse error at element `at`
    int64_t at = 0;
};

// A separator run before element k > 0 is valid when no ',' follows a tab,
// vertical tab or form feed in it (the skip stops at the first of those and
// scanf's white-space skip cannot pass a ','); before element 0 it may hold
// white space only.
inline bool run_ok(const unsigned char* b, int64_t lo, int64_t hi, bool first) {
    bool past_skip = first;
    for (int64_t p = lo; p < hi; ++p) {
        const unsigned char c = b[p];
        if (c == ',' && past_skip) return false;
        if (!is_skip(c)) past_skip = true;
    }
    return true;
}

// [+-]?digits, the whole token, within int64
inline bool fast_i64(const unsigned char* s, int64_t n, int64_t* out) {
    int64_t p = 0;
    bool neg = false;
    if (p < n && (s[p] == '+' || s[p] == '-')) neg = s[p++] == '-';
    if (p >= n) return false;
    unsigned long long v = 0;
    const unsigned long long lim = neg ? 9223372036854775808ULL : 9223372036854775807ULL;
    for (; p < n; ++p) {
        const unsigned d = (unsigned)s[p] - '0';
        if (d > 9) return false;
        if (v > (lim - d) / 10) return false;  // out of range: the sequential pass decides
        v = v * 10 + d;
    }
    *out = neg ? (int64_t)(0ULL - v) : (int64_t)v;
    return true;
}

// [+-]?(digits[.digits?] | .digits)([eE][+-]?digits)?, the whole token
inline bool fast_f64_form(const unsigned char* s, int64_t n) {
    int64_t p = 0;
    if (p < n && (s[p] == '+' || s[p] == '-')) ++p;
    int64_t digits = 0;
    while (p < n && s[p] >= '0' && s[p] <= '9') ++p, ++digits;
    if (p < n && s[p] == '.') {
        ++p;
        while (p < n && s[p] >= '0' && s[p] <= '9') ++p, ++digits;
    }
    if (digits == 0) return false;
    if (p < n && (s[p] == 'e' || s[p] == 'E')) {
        ++p;
        if (p < n && (s[p] == '+' || s[p] == '-')) ++p;
        int64_t ed = 0;
        while (p < n && s[p] >= '0' && s[p] <= '9') ++p, ++ed;
        if (ed == 0) return false;
    }
    return p == n;
}

template <class T>
bool fast_token(const unsigned char* s, int64_t n, T* out) {
    if constexpr (sizeof(T) == 8 && std::is_integral<T>::value) {
        return fast_i64(s, n, out);
    } else {
        if (!fast_f64_form(s, n) || n > 400) return false;
        char tmp[416];
        memcpy(tmp, s, (size_t)n);
        tmp[n] = '\0';
        *out = strtod(tmp, nullptr);
        return true;
    }
}

// The sequential pass: the reference's loop, each conversion by sscanf on a
// copy of the token (a number never spans ',' or white space, so the copy
// ends where the stream would offer scanf a non-number character).
template <class T>
CsvError read_exact(const unsigned char* b, int64_t len, int64_t size, T* out) {
    CsvError e;
    int64_t pos = 0;
    std::string tok;
    for (int64_t i = 0; i < size; ++i) {
        if (i > 0) {
            while (pos < len && is_skip(b[pos])) ++pos;
            if (pos >= len) return CsvError{1, i};
        }
        int64_t q = pos;
        while (q < len && is_ws(b[q])) ++q;
        if (q >= len) return CsvError{2, i};
        int64_t end = q;
        while (end < len && !is_sep(b[end])) ++end;
        tok.assign(reinterpret_cast<const char*>(b + q), (size_t)(end - q));
        int used = 0;
        int got;
        if constexpr (std::is_integral<T>::value) {
            long long v = 0;
            got = sscanf(tok.c_str(), "%lld%n", &v, &used);
            if (got == 1) out[i] = (T)v;
        } else {
            double v = 0.0;
            got = sscanf(tok.c_str(), "%lf%n", &v, &used);
            if (got == 1) out[i] = (T)v;
        }
        if (got != 1) return CsvError{2, i};
        pos = q + used;
    }
    return e;
}

struct Slice {
    int64_t lo, hi;            // byte range, starting at a token start (or 0)
    std::vector<double> f;     // values (one of the two is used)
    std::vector<int64_t> ints;
    int64_t count = 0;         // tokens in the range
    int64_t first_bad = -1;    // index (within the range) of the first token the fast path refused
    int64_t last_end = 0;      // end of the range's last token
};

template <class T>
void parse_slice(const unsigned char* b, int64_t len, Slice& s) {
    std::vector<T>& vals = [&]() -> std::vector<T>& {
        if constexpr (std::is_integral<T>::value) return s.ints;
        else return s.f;
    }();
    int64_t p = s.lo;
    while (p < s.hi) {
        while (p < s.hi && is_sep(b[p])) ++p;
        if (p >= s.hi) break;
        int64_t end = p;
        while (end < len && !is_sep(b[end])) ++end;
        // the separator run before this token; it is the file's first token
        // when nothing but separators precedes it
        int64_t r = p;
        while (r > 0 && is_sep(b[r - 1])) --r;
        T v{};
        const bool ok = run_ok(b, r, p, r == 0) && fast_token<T>(b + p, end - p, &v);
        if (!ok && s.first_bad < 0) s.first_bad = s.count;
        vals.push_back(v);
        ++s.count;
        s.last_end = end;
        p = end;
    }
}

template <class T>
CsvError read_parallel(const unsigned char* b, int64_t len, int64_t size, T* out) {
    if (size <= 0) return CsvError{};
    unsigned nt = std::thread::hardware_concurrency();
    if (nt == 0) nt = 1;
    const int64_t per = (int64_t)1 << 20;  // at least 1 MiB of text per thread
    if ((int64_t)nt > len / per + 1) nt = (unsigned)(len / per + 1);
    if (nt > 64) nt = 64;
    std::vector<Slice> sl(nt);
    for (unsigned t = 0; t < nt; ++t) {
        int64_t lo = len * t / nt;
        // move to a token start (the previous character a separator)
        if (t > 0) {
            while (lo < len && !(is_sep(b[lo - 1]) && !is_sep(b[lo]))) ++lo;
        }
        sl[t].lo = lo;
    }
    for (unsigned t = 0; t < nt; ++t) sl[t].hi = t + 1 < nt ? sl[t + 1].lo : len;
    for (unsigned t = 0; t + 1 < nt; ++t)
        if (sl[t].hi < sl[t].lo) sl[t].hi = sl[t].lo;
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; ++t) th.emplace_back([&, t] { parse_slice<T>(b, len, sl[t]); });
    parse_slice<T>(b, len, sl[0]);
    for (auto& x : th) x.join();
    // element index of each slice's first token; the first refused token
    int64_t base = 0, bad = -1, total = 0, last_end = 0;
    std::vector<int64_t> start(nt);
    for (unsigned t = 0; t < nt; ++t) {
        start[t] = base;
        if (bad < 0 && sl[t].first_bad >= 0) bad = base + sl[t].first_bad;
        base += sl[t].count;
        if (sl[t].count) last_end = sl[t].last_end;
    }
    total = base;
    if (bad >= 0 && bad < size) return read_exact<T>(b, len, size, out);
    if (total < size) {
        // what the reference meets after the last token: the skip reaching the
        // end ("too few values"), or white space it leaves to scanf, which
        // then meets the end or a ',' (a parse error)
        if (total == 0) return CsvError{2, 0};
        int64_t p = last_end;
        while (p < len && is_skip(b[p])) ++p;
        return p >= len ? CsvError{1, total} : CsvError{2, total};
    }
    std::vector<std::thread> cp;
    for (unsigned t = 0; t < nt; ++t) {
        const int64_t lo = start[t], n = sl[t].count;
        if (lo >= size || n == 0) continue;
        const int64_t m = lo + n <= size ? n : size - lo;
        cp.emplace_back([&, t, lo, m] {
            if constexpr (std::is_integral<T>::value) memcpy(out + lo, sl[t].ints.data(), (size_t)m * sizeof(T));
            else memcpy(out + lo, sl[t].f.data(), (size_t)m * sizeof(T));
        });
    }
    for (auto& x : cp) x.join();
    return CsvError{};
}

// The whole file in memory; false when it cannot be opened or read.
bool slurp(const char* path, std::vector<unsigned char>& buf) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    buf.clear();
    if (fseek(f, 0, SEEK_END) == 0) {
        const long sz = ftell(f);
        if (sz > 0) {
            buf.resize((size_t)sz);
            rewind(f);
            const size_t got = fread(buf.data(), 1, (size_t)sz, f);
            buf.resize(got);
            fclose(f);
            return true;
        }
        rewind(f);
    }
    unsigned char chunk[1 << 16];  // streams without a size
    size_t got;
    while ((got = fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    fclose(f);
    return true;
}

int64_t shape_elems(const hyd_tuple_t& s) {
    int64_t n = 1;
    for (int i = 0; i < s.ndims; ++i) n *= s.elems[i];
    return n;
}

// The rows of the output, formatted on all host threads, in order.
template <class T>
std::string format_rows(const T* v, int ndims, const hyd_tuple_t& shape) {
    const int64_t size = shape_elems(shape);
    const int64_t rows = ndims == 2 ? shape.elems[0] : 1;
    const int64_t cols = ndims == 2 ? shape.elems[1] : size;
    unsigned nt = std::thread::hardware_concurrency();
    if (nt == 0) nt = 1;
    const int64_t cells = rows * (cols > 0 ? cols : 1);
    if ((int64_t)nt > cells / 65536 + 1) nt = (unsigned)(cells / 65536 + 1);
    if (nt > 64) nt = 64;
    std::vector<std::string> part(nt);
    auto work = [&](unsigned t) {
        // cells [c0, c1) in row-major order; a row of zero columns is one "\n"
        const int64_t c0 = cells * t / nt, c1 = cells * (t + 1) / nt;
        std::string& o = part[t];
        o.reserve((size_t)(c1 - c0) * 24);
        char tmp[64];
        for (int64_t c = c0; c < c1; ++c) {
            if (cols == 0) {
                o.push_back('\n');
                continue;
            }
            const int64_t j = c % cols;
            if (j) o.push_back(',');
            int k;
            if constexpr (std::is_integral<T>::value) k = snprintf(tmp, sizeof tmp, "%lld", (long long)v[c]);
            else k = snprintf(tmp, sizeof tmp, "%.17g", (double)v[c]);
            o.append(tmp, (size_t)k);
            if (j == cols - 1) o.push_back('\n');
        }
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& x : th) x.join();
    std::string all;
    size_t bytes = 0;
    for (auto& p : part) bytes += p.size();
    all.reserve(bytes);
    for (auto& p : part) all += p;
    return all;
}

bool write_text(const char* path, const std::string& text) {
    FILE* f = fopen(path, "w");
    if (!f) return false;
    const bool ok = fwrite(text.data(), 1, text.size(), f) == text.size();
    return fclose(f) == 0 && ok;
}

template <class T>
hyd_array_t* read_host(const char* path, hyd_tuple_t shape, const char* who) {
    std::vector<unsigned char> buf;
    if (!slurp(path, buf)) {
        fprintf(stderr, "%s: cannot open '%s'\n", who, path);
        exit(1);
    }
    hyd_array_t* a = hyd_cuda_array_alloc(shape, 8);  // what the reference's hyd_array_free releases
    if (!a) {
        fprintf(stderr, "%s: out of memory\n", who);
        exit(1);
    }
    const CsvError e = read_parallel<T>(buf.data(), (int64_t)buf.size(), shape_elems(shape), (T*)a->data);
    if (e.kind == 1) {
        fprintf(stderr, "%s: too few values\n", who);
        exit(1);
    }
    if (e.kind == 2) {
        fprintf(stderr, "%s: parse error at element %lld\n", who, (long long)e.at);
        exit(1);
    }
    return a;
}

template <class T>
int read_device(const char* path, int64_t n, void* dev, void* stream, const char* who) {
    HYD_CHECK_ARG(path != nullptr && n >= 0 && (n == 0 || dev != nullptr), "%s: bad arguments", who);
    std::vector<unsigned char> buf;
    if (!slurp(path, buf)) return set_error(HYD_CUDA_ERR_INVALID, "%s: cannot open '%s'", who, path);
    if (n == 0) return HYD_CUDA_OK;
    T* pinned = nullptr;
    HYD_CUDA_TRY(cudaHostAlloc((void**)&pinned, (size_t)n * sizeof(T), cudaHostAllocDefault));
    const CsvError e = read_parallel<T>(buf.data(), (int64_t)buf.size(), n, pinned);
    int st = HYD_CUDA_OK;
    if (e.kind == 1) st = set_error(HYD_CUDA_ERR_INVALID, "%s: too few values", who);
    else if (e.kind == 2) st = set_error(HYD_CUDA_ERR_INVALID, "%s: parse error at element %lld", who, (long long)e.at);
    cudaStream_t s = as_stream(stream);
    if (st == HYD_CUDA_OK && cudaMemcpyAsync(dev, pinned, (size_t)n * sizeof(T), cudaMemcpyHostToDevice, s) != cudaSuccess)
        st = set_error(HYD_CUDA_ERR_CUDA, "%s: copy to the device failed", who);
    if (st == HYD_CUDA_OK && cudaStreamSynchronize(s) != cudaSuccess)
        st = set_error(HYD_CUDA_ERR_CUDA, "%s: synchronize failed", who);
    cudaFreeHost(pinned);
    return st;
}

template <class T>
int write_device(const void* dev, hyd_tuple_t shape, const char* path, void* stream, const char* who) {
    HYD_CHECK_ARG(path != nullptr && shape.ndims >= 0 && shape.ndims <= 8, "%s: bad arguments", who);
    const int64_t n = shape_elems(shape);
    HYD_CHECK_ARG(n >= 0 && (n == 0 || dev != nullptr), "%s: bad shape or null data", who);
    T* pinned = nullptr;
    if (n) {
        HYD_CUDA_TRY(cudaHostAlloc((void**)&pinned, (size_t)n * sizeof(T), cudaHostAllocDefault));
        cudaStream_t s = as_stream(stream);
        if (cudaMemcpyAsync(pinned, dev, (size_t)n * sizeof(T), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            cudaFreeHost(pinned);
            return set_error(HYD_CUDA_ERR_CUDA, "%s: copy from the device failed", who);
        }
    }
    const bool ok = write_text(path, format_rows<T>(pinned, shape.ndims, shape));
    if (pinned) cudaFreeHost(pinned);
    return ok ? HYD_CUDA_OK : set_error(HYD_CUDA_ERR_INVALID, "%s: cannot write '%s'", who, path);
}

}  // namespace

}  // namespace hyd

using namespace hyd;

extern "C" {

hyd_array_t* hyd_cuda_read_array_csv(const char* filename, hyd_tuple_t shape) {
    return read_host<int64_t>(filename, shape, "read_array");
}

hyd_array_t* hyd_cuda_read_float_array_csv(const char* filename, hyd_tuple_t shape) {
    return read_host<double>(filename, shape, "read_array_float");
}

int64_t hyd_cuda_write_array_csv(hyd_array_t* arr, const char* filename) {
    const std::string text = format_rows<int64_t>((const int64_t*)arr->data, arr->shape.ndims, arr->shape);
    if (!write_text(filename, text)) {
        perror("fopen");
        exit(1);
    }
    return 0;
}

int64_t hyd_cuda_write_array_csv_float(hyd_array_t* arr, const char* filename) {
    const std::string text = format_rows<double>((const double*)arr->data, arr->shape.ndims, arr->shape);
    if (!write_text(filename, text)) {
        perror("fopen");
        exit(1);
    }
    return 0;
}

int hyd_cuda_read_csv_i64_to_device(const char* filename, int64_t n, int64_t* dev, void* stream) {
    return read_device<int64_t>(filename, n, dev, stream, "read_csv_i64_to_device");
}

int hyd_cuda_read_csv_f64_to_device(const char* filename, int64_t n, double* dev, void* stream) {
    return read_device<double>(filename, n, dev, stream, "read_csv_f64_to_device");
}

int hyd_cuda_write_csv_i64_from_device(const int64_t* dev, hyd_tuple_t shape, const char* filename, void* stream) {
    return write_device<int64_t>(dev, shape, filename, stream, "write_csv_i64_from_device");
}

int hyd_cuda_write_csv_f64_from_device(const double* dev, hyd_tuple_t shape, const char* filename, void* stream) {
    return write_device<double>(dev, shape, filename, stream, "write_csv_f64_from_device");
}

}  // extern "C"
