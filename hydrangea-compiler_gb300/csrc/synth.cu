// synth.cu -- seeded synthetic inputs for the batched COO -> CSR -> SpMV
// workload (512 instances of uneven size).  Test/benchmark input generation,
// not part of any hot path.
//
// Instance i uses seed s = seed0 + i and the counter-based SplitMix64 stream
// (element k of a stream depends only on (s, k)):
//   n        = floor(2^(min_log2 + (max_log2 - min_log2) * u)), u = U[0,1) (stream 0)
//   len(r)   ~ Zipf(1.5) on {1..max_row_len} by inverse CDF (stream 1 + r);
//              the CDF table is built from 1/(k*sqrt(k)) with IEEE-exact ops,
//              identical on every machine
//   cols(r)  = (start_r + j * p_r) mod n, j < len(r): distinct because the
//              stride p_r is a prime above 2^18 >= n (streams 2^40 + r, 2^41 + r)
//   vals     = U[-1,1) per row-major entry q (stream 2^42 + q)
//   x        = U[-1,1) per column (stream 2^43 + c)
//   COO order: row-major entry q is stored at position p = a^-1 (q - b) mod nnz
//              (an affine permutation, a prime not dividing nnz), i.e. the
//              entries arrive shuffled and with no duplicate (row, col).
#include <cmath>
#include <vector>

#include "hyd_common.cuh"

namespace hyd {

int scan_i64_launch(const long long* in, long long* out, int64_t n, long long init, bool reverse,
                    bool inclusive, cudaStream_t stream);

constexpr unsigned long long kStrideBase = 1ULL << 40;
constexpr unsigned long long kStartBase = 1ULL << 41;
constexpr unsigned long long kValBase = 1ULL << 42;
constexpr unsigned long long kXBase = 1ULL << 43;
// primes above 2^18 (strides for distinct columns)
__constant__ unsigned long long c_primes[8] = {262147ULL, 262151ULL, 262153ULL, 262187ULL,
                                              262193ULL, 262217ULL, 262231ULL, 262237ULL};
__constant__ double c_zipf_cdf[257];  // cumulative weights, c_zipf_cdf[k] = sum_{j<=k} w_j

__device__ __forceinline__ double u01(uint64_t smix, uint64_t k) {
    return (double)(rand_u64(smix, k) >> 11) * 0x1.0p-53;
}

struct SynthInst {
    long long n, row_base, entry_base, nnz, a_inv, b;
    unsigned long long smix;
};

__device__ __forceinline__ int find_inst(const SynthInst* inst, int ninst, long long g) {
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst[mid].row_base <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int zipf_len(double u, int maxlen) {
    const double t = u * c_zipf_cdf[maxlen];
    int lo = 1, hi = maxlen;
    while (lo < hi) {  // smallest k with cdf[k] > t
        const int mid = (lo + hi) >> 1;
        if (c_zipf_cdf[mid] > t) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

__global__ void synth_row_len_kernel(const SynthInst* __restrict__ inst, int ninst, long long rows_total,
                                     int maxlen, long long* __restrict__ len) {
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < rows_total;
         g += (long long)gridDim.x * blockDim.x) {
        const int i = find_inst(inst, ninst, g);
        const long long r = g - inst[i].row_base;
        len[g] = zipf_len(u01(inst[i].smix, 1ULL + (unsigned long long)r), maxlen);
    }
}

__global__ void synth_fill_kernel(const SynthInst* __restrict__ inst, int ninst, long long rows_total,
                                  const long long* __restrict__ len, const long long* __restrict__ row_off,
                                  int* __restrict__ rows, int* __restrict__ cols, double* __restrict__ vals) {
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < rows_total;
         g += (long long)gridDim.x * blockDim.x) {
        const int i = find_inst(inst, ninst, g);
        const SynthInst I = inst[i];
        const long long r = g - I.row_base;
        const unsigned long long n = (unsigned long long)I.n;
        const unsigned long long start = rand_u64(I.smix, kStartBase + r) % n;
        const unsigned long long p = c_primes[rand_u64(I.smix, kStrideBase + r) & 7] % n;
        const long long q0 = row_off[g] - row_off[I.row_base];  // row-major entry index in the instance
        const long long L = len[g];
        const unsigned long long nnz = (unsigned long long)I.nnz;
        for (long long j = 0; j < L; ++j) {
            const unsigned long long q = (unsigned long long)(q0 + j);
            const unsigned long long c = (start + (unsigned long long)j * p) % n;
            // position p = a_inv * (q - b) mod nnz  (q, b < nnz < 2^32: products fit 64 bits)
            const unsigned long long pos = ((q + nnz - (unsigned long long)I.b % nnz) % nnz) *
                                           (unsigned long long)I.a_inv % nnz;
            const long long e = I.entry_base + (long long)pos;
            rows[e] = (int)r;
            cols[e] = (int)c;
            vals[e] = __dadd_rn(-1.0, __dmul_rn(2.0, u01(I.smix, kValBase + q)));
        }
    }
}

__global__ void synth_x_kernel(const SynthInst* __restrict__ inst, int ninst, long long rows_total, double* __restrict__ x) {
    // square instances: x of instance i has n entries, concatenated like the rows
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < rows_total;
         g += (long long)gridDim.x * blockDim.x) {
        const int i = find_inst(inst, ninst, g);
        const long long c = g - inst[i].row_base;
        x[g] = __dadd_rn(-1.0, __dmul_rn(2.0, u01(inst[i].smix, kXBase + (unsigned long long)c)));
    }
}

static long long modinv(long long a, long long m) {  // a^-1 mod m, gcd(a, m) = 1
    long long t = 0, nt = 1, r = m, nr = a % m;
    while (nr != 0) {
        const long long q = r / nr;
        long long tmp = t - q * nt; t = nt; nt = tmp;
        tmp = r - q * nr; r = nr; nr = tmp;
    }
    return t < 0 ? t + m : t;
}

}  // namespace hyd

using namespace hyd;

extern "C" int hyd_cuda_synth_coo_batch(int64_t ninst, uint64_t seed0, int min_log2, int max_log2, int max_row_len,
                                        int64_t* desc, int32_t* rows, int32_t* cols, double* vals, double* x,
                                        int64_t capacity_entries, void* stream) {
    HYD_CHECK_ARG(ninst > 0 && ninst < (1 << 20), "synth_coo_batch: bad instance count");
    HYD_CHECK_ARG(min_log2 >= 1 && max_log2 >= min_log2 && max_log2 <= 20, "synth_coo_batch: log2 range in [1, 20]");
    HYD_CHECK_ARG(max_row_len >= 1 && max_row_len <= 256 && (1 << min_log2) >= max_row_len,
                  "synth_coo_batch: max_row_len in [1, 256] and <= 2^min_log2");
    HYD_CHECK_ARG(desc != nullptr, "synth_coo_batch: null desc");
    cudaStream_t s = as_stream(stream);
    Device* d = nullptr;
    HYD_TRY(device(&d));
    // Zipf(1.5) CDF from IEEE-exact operations (sqrt, mul, div, add are correctly rounded)
    double cdf[257];
    cdf[0] = 0.0;
    for (int k = 1; k <= 256; ++k) cdf[k] = cdf[k - 1] + 1.0 / ((double)k * std::sqrt((double)k));
    HYD_CUDA_TRY(cudaMemcpyToSymbolAsync(c_zipf_cdf, cdf, sizeof cdf, 0, cudaMemcpyHostToDevice, s));
    std::vector<SynthInst> inst((size_t)ninst);
    long long rows_total = 0;
    for (int64_t i = 0; i < ninst; ++i) {
        const unsigned long long smix = mix64(seed0 + (unsigned long long)i);
        const double u = (double)(rand_u64(smix, 0) >> 11) * 0x1.0p-53;
        long long n = (long long)std::floor(std::exp2((double)min_log2 + (double)(max_log2 - min_log2) * u));
        if (n < (1LL << min_log2)) n = 1LL << min_log2;
        inst[i] = SynthInst{n, rows_total, 0, 0, 1, 0, smix};
        rows_total += n;
    }
    void* buf = nullptr;
    const size_t inst_bytes = ((size_t)ninst * sizeof(SynthInst) + 255) & ~(size_t)255;
    const size_t row_bytes = ((size_t)rows_total * 8 + 255) & ~(size_t)255;
    HYD_TRY(device_buffer(d, "synth_tables", inst_bytes + 2 * row_bytes, &buf));
    SynthInst* d_inst = static_cast<SynthInst*>(buf);
    long long* len = reinterpret_cast<long long*>(static_cast<unsigned char*>(buf) + inst_bytes);
    long long* off = len + row_bytes / 8;
    HYD_CUDA_TRY(cudaMemcpyAsync(d_inst, inst.data(), inst.size() * sizeof(SynthInst), cudaMemcpyHostToDevice, s));
    const unsigned grid = (unsigned)(d->sm_count * 8);
    synth_row_len_kernel<<<grid, 256, 0, s>>>(d_inst, (int)ninst, rows_total, max_row_len, len);
    HYD_TRY(launch_check("synth_row_len"));
    HYD_TRY(scan_i64_launch(len, off, rows_total, 0, false, false, s));
    // per-instance nnz = off[next row_base] - off[row_base]
    std::vector<long long> first((size_t)ninst), last_len(1);
    for (int64_t i = 0; i < ninst; ++i)
        HYD_CUDA_TRY(cudaMemcpyAsync(&first[i], off + inst[i].row_base, 8, cudaMemcpyDeviceToHost, s));
    long long last_off = 0;
    HYD_CUDA_TRY(cudaMemcpyAsync(&last_off, off + rows_total - 1, 8, cudaMemcpyDeviceToHost, s));
    HYD_CUDA_TRY(cudaMemcpyAsync(&last_len[0], len + rows_total - 1, 8, cudaMemcpyDeviceToHost, s));
    HYD_CUDA_TRY(cudaStreamSynchronize(s));
    const long long total = last_off + last_len[0];
    for (int64_t i = 0; i < ninst; ++i) {
        const long long nz = (i + 1 < ninst ? first[i + 1] : total) - first[i];
        inst[i].entry_base = first[i];
        inst[i].nnz = nz;
        // affine shuffle: a prime that does not divide nnz
        static const long long primes[4] = {1000003LL, 998244353LL, 1000000007LL, 754974721LL};
        long long a = primes[0];
        for (long long pr : primes)
            if (nz % pr != 0) { a = pr; break; }
        inst[i].a_inv = nz > 1 ? modinv(a % nz, nz) : 0;
        inst[i].b = nz > 0 ? (long long)(rand_u64(inst[i].smix, 3) % (unsigned long long)nz) : 0;
        desc[3 * i] = inst[i].n;
        desc[3 * i + 1] = inst[i].n;
        desc[3 * i + 2] = nz;
    }
    if (rows == nullptr) return HYD_CUDA_OK;  // sizes only
    HYD_CHECK_ARG(cols && vals && x, "synth_coo_batch: null output");
    HYD_CHECK_ARG(capacity_entries >= total, "synth_coo_batch: capacity %lld < %lld entries",
                  (long long)capacity_entries, total);
    HYD_CUDA_TRY(cudaMemcpyAsync(d_inst, inst.data(), inst.size() * sizeof(SynthInst), cudaMemcpyHostToDevice, s));
    synth_fill_kernel<<<grid, 256, 0, s>>>(d_inst, (int)ninst, rows_total, len, off, rows, cols, vals);
    HYD_TRY(launch_check("synth_fill"));
    synth_x_kernel<<<grid, 256, 0, s>>>(d_inst, (int)ninst, rows_total, x);
    HYD_TRY(launch_check("synth_x"));
    HYD_CUDA_TRY(cudaStreamSynchronize(s));
    return HYD_CUDA_OK;
}
