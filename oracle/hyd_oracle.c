/* oracle/hyd_oracle.c -- CPU oracle for the Hydrangea fused-loop hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see hyd_oracle.h).  Every loop below restates the
 * shape that the reference C backend emits for one combinator, in the same
 * floating-point evaluation order, compiled with the backend's own flags
 * (-O3 -std=c99 -fopenmp; ISO C mode keeps FMA contraction off, which is what
 * app/CBackend.hs:89 gets too).  Integer arithmetic that the generated C does
 * in int64_t is done here in uint64_t so that wrap-around is defined.
 *
 * Reference paths are relative to the hydrangea-compiler source tree.
 */
#include "hyd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* Seeded counter-based generator.  SplitMix64's output function (Steele, Lea
 * and Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014)
 * applied to a Weyl sequence indexed by the element number, so element i of
 * a stream can be computed independently on any thread, CPU or GPU.           */
static inline uint64_t orc_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

uint64_t orc_rand_u64(uint64_t seed, uint64_t i) {
    return orc_mix64(orc_mix64(seed) + (i + 1ULL) * 0x9E3779B97F4A7C15ULL);
}

void orc_fill_uniform_f64(double* out, int64_t n, uint64_t seed, double lo, double hi) {
    const double scale = hi - lo;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double u = (double)(orc_rand_u64(seed, (uint64_t)i) >> 11) * 0x1.0p-53;
        double t = scale * u;
        out[i] = lo + t;
    }
}

void orc_fill_uniform_i64(int64_t* out, int64_t n, uint64_t seed, int64_t bound) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        out[i] = (int64_t)(orc_rand_u64(seed, (uint64_t)i) % (uint64_t)bound);
    }
}

/* ------------------------------------------------------------------------- */
/* reduce (+) 0.0 (zipwith (*) xs ys).
 * Fusion.hs:2141 (fuseReduce) turns the pair into one reduce_generate;
 * Lowering.hs:771-804 lowers it to a LoopReduction whose body is
 * `acc = acc + xs[i] * ys[i]`; CodegenC.hs:1328-1353 emits it as
 * `#pragma omp parallel for simd simdlen(4) reduction(+:acc)` (the simd clause
 * per CodegenC.hs:1050-1054; emitted text shown at README.md:25-33).         */
double orc_dot_f64(const double* xs, const double* ys, int64_t n) {
    double acc = 0.0;
#pragma omp parallel for simd simdlen(4) reduction(+:acc)
    for (int64_t i = 0; i < n; i++) {
        acc = acc + xs[i] * ys[i];
    }
    return acc;
}

/* The serial template of the same loop (CodegenC.hs:1306-1327). */
double orc_dot_f64_serial(const double* xs, const double* ys, int64_t n) {
    double acc = 0.0;
    for (int64_t i = 0; i < n; i++) {
        acc = acc + xs[i] * ys[i];
    }
    return acc;
}

/* FP64 truth: each product split exactly into hi+lo with the Dekker/Veltkamp
 * two-product (no FMA needed), then every term accumulated with Neumaier's
 * compensated summation.  Error is O(eps) relative to sum |x*y| instead of
 * O(n eps).                                                                  */
static inline void orc_two_prod(double a, double b, double* p, double* e) {
    const double split = 134217729.0; /* 2^27 + 1 */
    double x = a * b;
    double ca = split * a, cb = split * b;
    double ahi = ca - (ca - a), alo = a - ahi;
    double bhi = cb - (cb - b), blo = b - bhi;
    *p = x;
    *e = ((ahi * bhi - x) + ahi * blo + alo * bhi) + alo * blo;
}

static inline void orc_neumaier_add(double* s, double* c, double v) {
    double t = *s + v;
    if (fabs(*s) >= fabs(v)) {
        *c += (*s - t) + v;
    } else {
        *c += (v - t) + *s;
    }
    *s = t;
}

double orc_dot_f64_compensated(const double* xs, const double* ys, int64_t n) {
    double s = 0.0, c = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double p, e;
        orc_two_prod(xs[i], ys[i], &p, &e);
        orc_neumaier_add(&s, &c, p);
        orc_neumaier_add(&s, &c, e);
    }
    return s + c;
}

double orc_sum_f64_compensated(const double* xs, int64_t n) {
    double s = 0.0, c = 0.0;
    for (int64_t i = 0; i < n; i++) {
        orc_neumaier_add(&s, &c, xs[i]);
    }
    return s + c;
}

/* ------------------------------------------------------------------------- */
/* Fused element chains.  Fusion composes map/zipwith/generate chains into one
 * element function (Fusion.hs:1808-1874: map f (zipwith g xs ys) =>
 * zipwith (f . g), zipwith f (map g xs) ys => zipwith (\x y -> f (g x) y), ...)
 * and the C backend emits one `omp parallel for` over the elements with the
 * composed body (CodegenC.hs:1451-1491), or the reduction template when the
 * chain ends in reduce (+) (CodegenC.hs:1328-1353).  Two chains are restated:
 *
 * bench/map_chain/map_chain.hyd:11-17
 *   src = generate [n] (fn [i] => float_of i /. float_of n)
 *   c   = map (x *. 2.0 +. 1.0) (map (x -. 0.5) (map (x *. x) src))
 *   reduce (+.) 0.0 c
 * elements: ((s * s) - 0.5) * 2.0 + 1.0 with s = (double)i / (double)n.      */
static inline double orc_map_chain_elem(int64_t i, int64_t n) {
    const double s = (double)i / (double)n;
    const double a = s * s;
    const double b = a - 0.5;
    return b * 2.0 + 1.0;
}

void orc_map_chain_f64(int64_t n, double* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        out[i] = orc_map_chain_elem(i, n);
    }
}

/* The reduced form as the C backend runs it (reduction template). */
double orc_map_chain_sum_f64(int64_t n) {
    double acc = 0.0;
#pragma omp parallel for simd simdlen(4) reduction(+:acc)
    for (int64_t i = 0; i < n; i++) {
        acc = acc + orc_map_chain_elem(i, n);
    }
    return acc;
}

/* zipwith (+.) (zipwith ( *. ) a b) c, fused into one loop over three inputs:
 * out[i] = a[i] * b[i] + c[i], two IEEE roundings (no contraction).         */
void orc_zipwith_muladd_f64(const double* a, const double* b, const double* c, double* out, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        const double p = a[i] * b[i];
        out[i] = p + c[i];
    }
}

/* ------------------------------------------------------------------------- */
/* scatter (+) (fill [B] 0) (map (x % B) data) (map (x * x) data).
 * Fusion (scatter re-index, examples/weighted_histogram.hyd:1-25) reads data
 * once per element; Parallelize.hs:466-503 picks the privatized strategy when
 * the destination has at most 262144 cells (Parallelize.hs:492), and
 * CodegenC.hs:1119-1288 emits: an nthreads x B calloc grid, an `omp for`
 * accumulation into the calling thread's slice, and an `omp for` merge over
 * the cells that adds the slices in thread order (emitted text at
 * README.md:51-86).  `%` is C's truncating remainder (CodegenC.hs:2469-2474).
 * Returns 0, or -1 when a route leaves [0, B) (the generated C would write out
 * of bounds; the refinement checker is what normally rules that out).        */
#define ORC_PRIVATIZATION_CAP 262144

int orc_weighted_hist_i64(const int64_t* data, int64_t n, int64_t bins, int64_t* hist) {
    if (bins <= 0) return -1;
    if (bins > ORC_PRIVATIZATION_CAP) return orc_weighted_hist_i64_atomic(data, n, bins, hist);
    int nthr = orc_max_threads();
    uint64_t* grids = (uint64_t*)calloc((size_t)nthr * (size_t)bins, sizeof(uint64_t));
    if (grids == NULL) return -2;
    int bad = 0;
#pragma omp parallel
    {
        int tid = 0, nt = 1;
#ifdef _OPENMP
        tid = omp_get_thread_num();
        nt = omp_get_num_threads();
#endif
        uint64_t* priv = grids + (size_t)tid * (size_t)bins;
#pragma omp for
        for (int64_t i = 0; i < n; i++) {
            int64_t x = data[i];
            int64_t bin = x % bins;
            uint64_t val = (uint64_t)x * (uint64_t)x;
            if (bin < 0 || bin >= bins) {
                bad = 1;
                continue;
            }
            priv[bin] += val;
        }
#pragma omp for
        for (int64_t b = 0; b < bins; b++) {
            uint64_t sum = (uint64_t)hist[b];
            for (int t = 0; t < nt; t++) {
                sum += grids[(size_t)t * (size_t)bins + b];
            }
            hist[b] = (int64_t)sum;
        }
    }
    free(grids);
    return bad ? -1 : 0;
}

/* The atomic template (CodegenC.hs:1084-1118): `#pragma omp atomic update`
 * on the destination cell, used above the privatization cap.                */
int orc_weighted_hist_i64_atomic(const int64_t* data, int64_t n, int64_t bins, int64_t* hist) {
    if (bins <= 0) return -1;
    int bad = 0;
    uint64_t* h = (uint64_t*)hist;
#pragma omp parallel for
    for (int64_t i = 0; i < n; i++) {
        int64_t x = data[i];
        int64_t bin = x % bins;
        uint64_t val = (uint64_t)x * (uint64_t)x;
        if (bin < 0 || bin >= bins) {
            bad = 1;
            continue;
        }
#pragma omp atomic update
        h[bin] += val;
    }
    return bad ? -1 : 0;
}

/* bench/weighted_histogram/weighted_histogram.hyd: bucket [i] = (i*bins)/n,
 * weight [i] = i*3 + 1, scattered with (+) into fill [bins] 0 (privatized as
 * above).                                                                   */
int orc_hist_generate_i64(int64_t n, int64_t bins, int64_t* hist) {
    if (bins <= 0 || n <= 0) return -1;
    int nthr = orc_max_threads();
    uint64_t* grids = (uint64_t*)calloc((size_t)nthr * (size_t)bins, sizeof(uint64_t));
    if (grids == NULL) return -2;
#pragma omp parallel
    {
        int tid = 0, nt = 1;
#ifdef _OPENMP
        tid = omp_get_thread_num();
        nt = omp_get_num_threads();
#endif
        uint64_t* priv = grids + (size_t)tid * (size_t)bins;
#pragma omp for
        for (int64_t i = 0; i < n; i++) {
            int64_t bucket = (i * bins) / n;
            uint64_t weight = (uint64_t)i * 3ULL + 1ULL;
            priv[bucket] += weight;
        }
#pragma omp for
        for (int64_t b = 0; b < bins; b++) {
            uint64_t sum = (uint64_t)hist[b];
            for (int t = 0; t < nt; t++) sum += grids[(size_t)t * (size_t)bins + b];
            hist[b] = (int64_t)sum;
        }
    }
    free(grids);
    return 0;
}

/* Unfused scatter (+) over materialised routes/values (Lowering.hs:1408-1430),
 * privatized under the cap, atomic above it.                                 */
int orc_scatter_add_i64(const int64_t* idx, const int64_t* vals, int64_t n,
                        int64_t* dst, int64_t dst_n) {
    int bad = 0;
    uint64_t* d = (uint64_t*)dst;
    if (dst_n > ORC_PRIVATIZATION_CAP) {
#pragma omp parallel for
        for (int64_t i = 0; i < n; i++) {
            int64_t b = idx[i];
            if (b < 0 || b >= dst_n) { bad = 1; continue; }
#pragma omp atomic update
            d[b] += (uint64_t)vals[i];
        }
        return bad ? -1 : 0;
    }
    int nthr = orc_max_threads();
    uint64_t* grids = (uint64_t*)calloc((size_t)nthr * (size_t)(dst_n > 0 ? dst_n : 1), sizeof(uint64_t));
    if (grids == NULL) return -2;
#pragma omp parallel
    {
        int tid = 0, nt = 1;
#ifdef _OPENMP
        tid = omp_get_thread_num();
        nt = omp_get_num_threads();
#endif
        uint64_t* priv = grids + (size_t)tid * (size_t)dst_n;
#pragma omp for
        for (int64_t i = 0; i < n; i++) {
            int64_t b = idx[i];
            if (b < 0 || b >= dst_n) { bad = 1; continue; }
            priv[b] += (uint64_t)vals[i];
        }
#pragma omp for
        for (int64_t b = 0; b < dst_n; b++) {
            uint64_t sum = d[b];
            for (int t = 0; t < nt; t++) sum += grids[(size_t)t * (size_t)dst_n + b];
            d[b] = sum;
        }
    }
    free(grids);
    return bad ? -1 : 0;
}

/* Float scatter-add.  The privatized float template merges slices in thread
 * order, so its result depends on the thread count; the checker therefore
 * uses the serial order (element order) and compares with a tolerance.       */
int orc_scatter_add_f64(const int64_t* idx, const double* vals, int64_t n,
                        double* dst, int64_t dst_n) {
    for (int64_t i = 0; i < n; i++) {
        int64_t b = idx[i];
        if (b < 0 || b >= dst_n) return -1;
        dst[b] = dst[b] + vals[i];
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* 2-D clamp stencils with the 5-point footprint.
 * Lowering.hs:2562-2661 (lowerSplitStencil2D) splits a clamp stencil whose
 * accesses have constant offsets into an interior loop with raw indices and
 * boundary strips whose indices are clamped to [0, n-1] (Lowering.hs:2102-2130
 * segments, genBnd1DVar Lowering.hs:2760-2790 clamp arithmetic); each region
 * is a LoopMap the backend emits as `omp parallel for`.  Per point the body is
 * the program text evaluated left to right (Parser.y:167-171 precedences).
 * a = acc (-1) 0, b = acc 1 0, c = acc 0 (-1), d = acc 0 1, e = acc 0 0.     */
static inline double orc_stencil_body(int kind, double a, double b, double c,
                                      double d, double e) {
    switch (kind) {
    case ORC_ST_LAPLACIAN:
        return a + b + c + d + (e * (-4.0));
    case ORC_ST_JACOBI:
        return (a + b + c + d) / 4.0;
    case ORC_ST_HEAT: {
        double lap = a + b + c + d - (4.0 * e);
        return e + 0.1 * lap;
    }
    case ORC_ST_HEAT_EXAMPLE:
    default:
        return (a + b + c + d + e) / 5.0;
    }
}

static inline int64_t orc_clamp(int64_t v, int64_t n) {
    if (v < 0) v = 0;
    if (v >= n) v = n - 1;
    return v;
}

static inline double orc_stencil_point_clamped(int kind, const double* in, int64_t h,
                                               int64_t w, int64_t i, int64_t j) {
    int64_t im = orc_clamp(i - 1, h), ip = orc_clamp(i + 1, h);
    int64_t jm = orc_clamp(j - 1, w), jp = orc_clamp(j + 1, w);
    return orc_stencil_body(kind, in[im * w + j], in[ip * w + j], in[i * w + jm],
                            in[i * w + jp], in[i * w + j]);
}

void orc_stencil2d_f64(int kind, const double* in, double* out, int64_t h, int64_t w) {
    if (h <= 0 || w <= 0) return;
    if (h >= 2 && w >= 2) {
        /* interior region: raw offsets, no clamp */
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t i = 1; i < h - 1; i++) {
            for (int64_t j = 1; j < w - 1; j++) {
                out[i * w + j] = orc_stencil_body(kind, in[(i - 1) * w + j], in[(i + 1) * w + j],
                                                  in[i * w + (j - 1)], in[i * w + (j + 1)],
                                                  in[i * w + j]);
            }
        }
        /* boundary strips: top and bottom rows, then left and right columns */
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < w; j++) {
            out[j] = orc_stencil_point_clamped(kind, in, h, w, 0, j);
            out[(h - 1) * w + j] = orc_stencil_point_clamped(kind, in, h, w, h - 1, j);
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 1; i < h - 1; i++) {
            out[i * w] = orc_stencil_point_clamped(kind, in, h, w, i, 0);
            out[i * w + (w - 1)] = orc_stencil_point_clamped(kind, in, h, w, i, w - 1);
        }
    } else {
        /* exact-size cases (n < total pad): every access clamped */
        for (int64_t i = 0; i < h; i++)
            for (int64_t j = 0; j < w; j++)
                out[i * w + j] = orc_stencil_point_clamped(kind, in, h, w, i, j);
    }
}

/* iterate n init step (Lowering.hs:840-858) with the ping-pong buffers that
 * hoistIterateAllocs introduces (CFGOpt.hs:795-810).  Returns which buffer
 * (0 or 1) holds the final state.                                           */
int orc_iterate_stencil2d_f64(int kind, double* buf0, double* buf1, int64_t h, int64_t w,
                              int64_t iters) {
    double* cur = buf0;
    double* nxt = buf1;
    for (int64_t t = 0; t < iters; t++) {
        orc_stencil2d_f64(kind, cur, nxt, h, w);
        double* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    return cur == buf0 ? 0 : 1;
}

/* Boundary conditions of `stencil` (Syntax.hs:416-426): per dimension, the
 * index an offset access reads, as genBnd1DVar computes it
 * (Lowering.hs:2762-2812):
 *   clamp   max(0, min(raw, n-1));
 *   wrap    raw - (raw / n) * n with C's truncating division, plus n when
 *           negative;
 *   mirror  period = 2 (n-1); r = raw - (raw / period) * period, plus period
 *           when negative; then period - r when r >= n (a fold-back that
 *           does not repeat the edge).  The reference divides by zero when
 *           n == 1; callers refuse that extent.
 * `constant` keeps the raw index; the caller reads the default instead when
 * it is out of range (in 2-D when either index is, genBnd2D
 * Lowering.hs:2842-2870).                                                    */
int64_t orc_bound_index(int64_t raw, int64_t n, int mode) {
    if (mode == ORC_BND_CLAMP) {
        int64_t bi = raw;
        if (raw < 0) bi = 0;
        if (bi >= n) bi = n - 1;
        return bi;
    }
    if (mode == ORC_BND_WRAP) {
        int64_t q = raw / n;
        int64_t bi = raw - q * n;
        if (bi < 0) bi = bi + n;
        return bi;
    }
    if (mode == ORC_BND_MIRROR) {
        int64_t period = 2 * (n - 1);
        int64_t q = raw / period;
        int64_t r = raw - q * period;
        if (r < 0) r = r + period;
        if (r >= n) r = period - r;
        return r;
    }
    return raw;
}

static int orc_bound_ok(int mode, int64_t n) { return !(mode == ORC_BND_MIRROR && n < 2); }

/* Sum of `acc d` over the offsets, int64, in offset order: the 1-D stencils
 * of StencilSpec.hs (`acc (-1)`, `acc 1`, `acc (-1) + acc 0 + acc 1`, ...).
 * Returns -1 for a mirror boundary on an extent of 1.                      */
int orc_stencil1d_offsets_i64(const int64_t* in, int64_t* out, int64_t n, const int64_t* offs, int noff,
                              int mode, int64_t fill) {
    if (!orc_bound_ok(mode, n)) return -1;
    for (int64_t i = 0; i < n; i++) {
        int64_t acc = 0;
        for (int k = 0; k < noff; k++) {
            int64_t raw = i + offs[k];
            int64_t v;
            if (mode == ORC_BND_CONST) v = (raw >= 0 && raw < n) ? in[raw] : fill;
            else v = in[orc_bound_index(raw, n, mode)];
            acc = (int64_t)((uint64_t)acc + (uint64_t)v);
        }
        out[i] = acc;
    }
    return 0;
}

/* 2-D form: offsets as (d0, d1) pairs; dimensions bounded independently,
 * `constant` reads the default when either index is out of range.           */
int orc_stencil2d_offsets_i64(const int64_t* in, int64_t* out, int64_t h, int64_t w, const int64_t* offs,
                              int noff, int mode, int64_t fill) {
    if (!orc_bound_ok(mode, h) || !orc_bound_ok(mode, w)) return -1;
    for (int64_t i = 0; i < h; i++)
        for (int64_t j = 0; j < w; j++) {
            int64_t acc = 0;
            for (int k = 0; k < noff; k++) {
                int64_t r0 = i + offs[2 * k], r1 = j + offs[2 * k + 1];
                int64_t v;
                if (mode == ORC_BND_CONST)
                    v = (r0 >= 0 && r0 < h && r1 >= 0 && r1 < w) ? in[r0 * w + r1] : fill;
                else
                    v = in[orc_bound_index(r0, h, mode) * w + orc_bound_index(r1, w, mode)];
                acc = (int64_t)((uint64_t)acc + (uint64_t)v);
            }
            out[i * w + j] = acc;
        }
    return 0;
}

/* The 5-point kinds of orc_stencil2d_f64 under any boundary condition: the
 * same body and evaluation order, neighbours read through orc_bound_index
 * (`constant`: `fill` out of range).  Returns -1 for a mirror boundary on an
 * extent of 1.  With ORC_BND_CLAMP it equals orc_stencil2d_f64.             */
int orc_stencil2d_bnd_f64(int kind, int mode, double fill, const double* in, double* out, int64_t h,
                          int64_t w) {
    if (!orc_bound_ok(mode, h) || !orc_bound_ok(mode, w)) return -1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t i = 0; i < h; i++)
        for (int64_t j = 0; j < w; j++) {
            double nb[4];
            const int64_t d0[4] = {-1, 1, 0, 0}, d1[4] = {0, 0, -1, 1};
            for (int k = 0; k < 4; k++) {
                int64_t r0 = i + d0[k], r1 = j + d1[k];
                if (mode == ORC_BND_CONST)
                    nb[k] = (r0 >= 0 && r0 < h && r1 >= 0 && r1 < w) ? in[r0 * w + r1] : fill;
                else
                    nb[k] = in[orc_bound_index(r0, h, mode) * w + orc_bound_index(r1, w, mode)];
            }
            out[i * w + j] = orc_stencil_body(kind, nb[0], nb[1], nb[2], nb[3], in[i * w + j]);
        }
    return 0;
}

int orc_iterate_stencil2d_bnd_f64(int kind, int mode, double fill, double* buf0, double* buf1, int64_t h,
                                  int64_t w, int64_t iters) {
    double* cur = buf0;
    double* nxt = buf1;
    for (int64_t t = 0; t < iters; t++) {
        if (orc_stencil2d_bnd_f64(kind, mode, fill, cur, nxt, h, w) != 0) return -1;
        double* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    return cur == buf0 ? 0 : 1;
}

/* `reduce` over the trailing axis (EReduce, Lowering.hs:723-760): for each
 * outer index j, acc = init; acc = acc op x[j*cols + k] for k in order;
 * out[j] = acc.  op 0: (+), 1: (*) (the Redop set, CFGCore.hs:236).  int64
 * arithmetic wraps.                                                          */
void orc_reduce_rows_i64(const int64_t* in, int64_t rows, int64_t cols, int op, int64_t init, int64_t* out) {
    for (int64_t j = 0; j < rows; j++) {
        uint64_t acc = (uint64_t)init;
        for (int64_t k = 0; k < cols; k++) {
            uint64_t x = (uint64_t)in[j * cols + k];
            acc = op == 0 ? acc + x : acc * x;
        }
        out[j] = (int64_t)acc;
    }
}

void orc_reduce_rows_f64(const double* in, int64_t rows, int64_t cols, int op, double init, double* out) {
    for (int64_t j = 0; j < rows; j++) {
        double acc = init;
        for (int64_t k = 0; k < cols; k++) {
            double x = in[j * cols + k];
            acc = op == 0 ? acc + x : acc * x;
        }
        out[j] = acc;
    }
}

/* A scatter (+) phase with a guard over materialised arrays (EScatterChain,
 * Lowering.hs:1768-1790): if guard[i] then dst[idx[i]] += vals[i].  Returns
 * -1 when a guarded index is out of range (the reference does not check).   */
int orc_scatter_add_guarded_i64(const int64_t* idx, const int64_t* vals, const int64_t* guard, int64_t n,
                                int64_t* dst, int64_t dst_n) {
    int bad = 0;
    for (int64_t i = 0; i < n; i++) {
        if (!guard[i]) continue;
        int64_t b = idx[i];
        if (b < 0 || b >= dst_n) {
            bad = 1;
            continue;
        }
        dst[b] = (int64_t)((uint64_t)dst[b] + (uint64_t)vals[i]);
    }
    return bad ? -1 : 0;
}

/* 1-D clamp 3-point box filter `acc (-1) + acc 0 + acc 1` (StencilSpec.hs:24-34). */
void orc_stencil1d_box3_i64(const int64_t* in, int64_t* out, int64_t n) {
    for (int64_t i = 0; i < n; i++) {
        int64_t l = orc_clamp(i - 1, n), r = orc_clamp(i + 1, n);
        out[i] = (int64_t)((uint64_t)in[l] + (uint64_t)in[i] + (uint64_t)in[r]);
    }
}

/* 1-D clamp Jacobi `stencil clamp (fn acc => (acc (-1) +. acc 0 +. acc 1) /. 3.0)`
 * (examples/jacobi_1d.hyd:4): the clamped split-region loop of
 * Lowering.hs:1932-2035 in one dimension; left-to-right sum, then the IEEE
 * division.                                                                  */
void orc_stencil1d_jacobi3_f64(const double* in, double* out, int64_t n) {
    for (int64_t i = 0; i < n; i++) {
        int64_t l = orc_clamp(i - 1, n), r = orc_clamp(i + 1, n);
        double s = in[l] + in[i];
        s = s + in[r];
        out[i] = s / 3.0;
    }
}

int orc_iterate_stencil1d_jacobi3_f64(double* buf0, double* buf1, int64_t n, int64_t iters) {
    double* cur = buf0;
    double* nxt = buf1;
    for (int64_t t = 0; t < iters; t++) {
        orc_stencil1d_jacobi3_f64(cur, nxt, n);
        double* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    return cur == buf0 ? 0 : 1;
}

/* One Gray-Scott step (demo/gray_scott/gray_scott.hyd:47-73): periodic
 * 5-point Laplacians of U and V through `imod`, the reaction terms, and the
 * updates, each expression evaluated left to right exactly as written:
 *   lap  = u[im1,j] + u[ip1,j] + u[i,jm1] + u[i,jp1] - 4*u_ij
 *   uvv  = u_ij * v_ij * v_ij
 *   u'   = u_ij + dt * (du*lap - uvv + feed*(1 - u_ij))
 *   v'   = v_ij + dt * (dv*lapv + uvv - (feed + kill)*v_ij)                  */
void orc_gray_scott_step_f64(const double* u, const double* v, double* un, double* vn, int64_t h, int64_t w,
                             double du, double dv, double feed, double kill, double dt) {
    for (int64_t i = 0; i < h; i++) {
        int64_t im1 = (i - 1 + h) % h, ip1 = (i + 1) % h;
        for (int64_t j = 0; j < w; j++) {
            int64_t jm1 = (j - 1 + w) % w, jp1 = (j + 1) % w;
            double uij = u[i * w + j], vij = v[i * w + j];
            double lu = u[im1 * w + j] + u[ip1 * w + j];
            lu = lu + u[i * w + jm1];
            lu = lu + u[i * w + jp1];
            lu = lu - 4.0 * uij;
            double lv = v[im1 * w + j] + v[ip1 * w + j];
            lv = lv + v[i * w + jm1];
            lv = lv + v[i * w + jp1];
            lv = lv - 4.0 * vij;
            double uvv = uij * vij;
            uvv = uvv * vij;
            double tu = du * lu;
            tu = tu - uvv;
            tu = tu + feed * (1.0 - uij);
            un[i * w + j] = uij + dt * tu;
            double tv = dv * lv;
            tv = tv + uvv;
            tv = tv - (feed + kill) * vij;
            vn[i * w + j] = vij + dt * tv;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* scan / scan_inclusive / scanr / scanr_inclusive with (+)
 * (Lowering.hs:3563-3612, lowerScanFamily): a serial LoopFold; the reverse
 * forms walk ix = n-1-k; the exclusive forms write the accumulator before the
 * step, the inclusive forms after it.                                        */
void orc_scan_i64(const int64_t* in, int64_t* out, int64_t n, int64_t init,
                  int reverse, int inclusive) {
    uint64_t acc = (uint64_t)init;
    for (int64_t k = 0; k < n; k++) {
        int64_t ix = reverse ? (n - 1 - k) : k;
        uint64_t elem = (uint64_t)in[ix];
        if (inclusive) {
            acc = acc + elem;
            out[ix] = (int64_t)acc;
        } else {
            out[ix] = (int64_t)acc;
            acc = acc + elem;
        }
    }
}

void orc_scan_f64(const double* in, double* out, int64_t n, double init,
                  int reverse, int inclusive) {
    double acc = init;
    for (int64_t k = 0; k < n; k++) {
        int64_t ix = reverse ? (n - 1 - k) : k;
        double elem = in[ix];
        if (inclusive) {
            acc = acc + elem;
            out[ix] = acc;
        } else {
            out[ix] = acc;
            acc = acc + elem;
        }
    }
}

/* segmented_reduce (+) init offsets vals (Lowering.hs:874-944): one output
 * per segment [offsets[s], offsets[s+1]), each accumulated left to right from
 * init; the outer loop is LoopSegRedOuter, emitted with schedule(dynamic)
 * (CodegenC.hs:1055-1057).  Returns -1 on offsets that leave [0, n_vals] or
 * decrease.                                                                 */
int orc_segmented_reduce_i64(const int64_t* offsets, int64_t n_offsets,
                             const int64_t* vals, int64_t n_vals, int64_t init,
                             int64_t* out) {
    int64_t nseg = n_offsets - 1;
    if (nseg < 0) return -1;
    int bad = 0;
#pragma omp parallel for schedule(dynamic)
    for (int64_t s = 0; s < nseg; s++) {
        int64_t start = offsets[s], stop = offsets[s + 1];
        if (start < 0 || stop > n_vals || stop < start) { bad = 1; continue; }
        uint64_t acc = (uint64_t)init;
        for (int64_t k = 0; k < stop - start; k++) acc = acc + (uint64_t)vals[start + k];
        out[s] = (int64_t)acc;
    }
    return bad ? -1 : 0;
}

int orc_segmented_reduce_f64(const int64_t* offsets, int64_t n_offsets,
                             const double* vals, int64_t n_vals, double init,
                             double* out) {
    int64_t nseg = n_offsets - 1;
    if (nseg < 0) return -1;
    int bad = 0;
#pragma omp parallel for schedule(dynamic)
    for (int64_t s = 0; s < nseg; s++) {
        int64_t start = offsets[s], stop = offsets[s + 1];
        if (start < 0 || stop > n_vals || stop < start) { bad = 1; continue; }
        double acc = init;
        for (int64_t k = 0; k < stop - start; k++) acc = acc + vals[start + k];
        out[s] = acc;
    }
    return bad ? -1 : 0;
}

/* ------------------------------------------------------------------------- */
/* sort_indices: the runtime's stable LSD radix sort of (key, index) entries
 * with 8-bit digits whose pass count comes from the largest key
 * (runtime/hydrangea_runtime.h:386-456).  The key digit is
 * (key >> shift) & 0xFF on the signed key, exactly as there.                 */
typedef struct { int64_t key; int64_t idx; } orc_entry_t;

void orc_sort_indices_i64(const int64_t* keys, int64_t n, int64_t* perm) {
    if (n <= 0) return;
    orc_entry_t* a = (orc_entry_t*)malloc((size_t)n * sizeof(orc_entry_t));
    orc_entry_t* b = (orc_entry_t*)malloc((size_t)n * sizeof(orc_entry_t));
    for (int64_t i = 0; i < n; i++) { a[i].key = keys[i]; a[i].idx = i; }
    int64_t max_key = 0;
    for (int64_t i = 0; i < n; i++) if (a[i].key > max_key) max_key = a[i].key;
    int passes = 0;
    for (int64_t mk = max_key; mk; mk >>= 8) passes++;
    if (passes == 0) passes = 1;
    orc_entry_t *src = a, *dst = b;
    for (int p = 0; p < passes; p++) {
        int shift = p * 8;
        int64_t count[256];
        memset(count, 0, sizeof(count));
        for (int64_t i = 0; i < n; i++) count[(src[i].key >> shift) & 0xFF]++;
        int64_t sum = 0;
        for (int j = 0; j < 256; j++) { int64_t c = count[j]; count[j] = sum; sum += c; }
        for (int64_t i = 0; i < n; i++) {
            int64_t d = (src[i].key >> shift) & 0xFF;
            dst[count[d]++] = src[i];
        }
        orc_entry_t* t = src; src = dst; dst = t;
    }
    for (int64_t i = 0; i < n; i++) perm[i] = src[i].idx;
    free(a);
    free(b);
}

/* gather perm src: out[i] = src[perm[i]] (a LoopMap over the permutation). */
void orc_gather_i64(const int64_t* perm, int64_t n, const int64_t* src, int64_t* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) out[i] = src[perm[i]];
}

void orc_gather_f64(const int64_t* perm, int64_t n, const double* src, double* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) out[i] = src[perm[i]];
}

/* coo_sum_duplicates (Lowering.hs:966-1080): one serial pass that keeps the
 * last written (row, col, val) in scalars and merges an entry into it when
 * both row and col repeat.  Returns the canonical count.                     */
int64_t orc_coo_sum_duplicates_i64(const int64_t* rows, const int64_t* cols,
                                   const int64_t* vals, int64_t nnz,
                                   int64_t* out_rows, int64_t* out_cols, int64_t* out_vals) {
    int64_t out_nnz = 0, prev_row = 0, prev_col = 0;
    uint64_t prev_val = 0;
    for (int64_t i = 0; i < nnz; i++) {
        int64_t row = rows[i], col = cols[i];
        uint64_t val = (uint64_t)vals[i];
        if (out_nnz > 0 && row == prev_row && col == prev_col) {
            prev_val = prev_val + val;
            out_vals[out_nnz - 1] = (int64_t)prev_val;
        } else {
            out_rows[out_nnz] = row;
            out_cols[out_nnz] = col;
            out_vals[out_nnz] = (int64_t)val;
            prev_row = row;
            prev_col = col;
            prev_val = val;
            out_nnz++;
        }
    }
    return out_nnz;
}

/* csr_from_sorted_coo (Lowering.hs:1081-1160): counts[row]++ per entry while
 * copying cols/vals through, then row_ptr[i] = running sum before row i and
 * row_ptr[nrows] = total.  Returns -1 on a row outside [0, nrows).          */
int orc_csr_from_sorted_coo_i64(int64_t nrows, int64_t nnz, const int64_t* rows,
                                const int64_t* cols, const int64_t* vals,
                                int64_t* row_ptr, int64_t* col_idx, int64_t* out_vals) {
    int64_t* counts = (int64_t*)calloc((size_t)(nrows > 0 ? nrows : 1), sizeof(int64_t));
    if (counts == NULL) return -2;
    for (int64_t i = 0; i < nnz; i++) {
        int64_t row = rows[i];
        if (row < 0 || row >= nrows) { free(counts); return -1; }
        counts[row] = counts[row] + 1;
        col_idx[i] = cols[i];
        out_vals[i] = vals[i];
    }
    int64_t acc = 0;
    for (int64_t i = 0; i < nrows; i++) {
        row_ptr[i] = acc;
        acc = acc + counts[i];
    }
    row_ptr[nrows] = acc;
    free(counts);
    return 0;
}

/* SpMV over CSR (bench/spmv/spmv.hyd:30-40): generate [nrows] of an inner
 * reduce_generate (+.) 0.0 [row_len] of values[k] *. x[col[k]], i.e. a
 * LoopMapReduction outer loop (`omp parallel for`) and a sequential inner sum
 * `acc = acc + v * x[c]` (Lowering.hs:771-838; the hand-written witness is
 * bench/spmv/spmv_ref.c:31-38).                                             */
void orc_spmv_csr_f64(int64_t nrows, const int64_t* row_ptr, const int64_t* col_idx,
                      const double* vals, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nrows; i++) {
        double acc = 0.0;
        int64_t start = row_ptr[i], len = row_ptr[i + 1] - row_ptr[i];
        for (int64_t k = 0; k < len; k++) {
            int64_t ka = k + start;
            acc = acc + vals[ka] * x[col_idx[ka]];
        }
        y[i] = acc;
    }
}

/* One instance of the batched float COO -> CSR -> SpMV program.
 * csr_from_sorted_coo is Int-only (Infer.hs:1825-1827), so the float-valued
 * build composes: packed key row*ncols+col (bench/coo_csr_build/
 * coo_csr_build.hyd:37-44) -> sort_indices -> gather rows/cols/vals ->
 * row counts by scatter (+) of ones -> exclusive scan of the counts
 * (scan (+) 0, with the total appended as row_ptr[nrows]) -> SpMV as above.
 * The synthetic instances carry no duplicate (row, col) pairs, so no
 * coo_sum_duplicates pass is needed.                                         */
int orc_coo_to_csr_spmv_f64(int64_t nrows, int64_t ncols, int64_t nnz,
                            const int32_t* rows, const int32_t* cols, const double* vals,
                            const double* x, int64_t* row_ptr, int32_t* col_idx,
                            double* csr_vals, double* y) {
    int64_t* keys = (int64_t*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
    int64_t* perm = (int64_t*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
    int64_t* counts = (int64_t*)calloc((size_t)(nrows > 0 ? nrows : 1), sizeof(int64_t));
    int64_t* cidx64 = (int64_t*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
    if (!keys || !perm || !counts || !cidx64) {
        free(keys); free(perm); free(counts); free(cidx64);
        return -2;
    }
    int bad = 0;
    for (int64_t i = 0; i < nnz; i++) {
        if (rows[i] < 0 || rows[i] >= nrows || cols[i] < 0 || cols[i] >= ncols) bad = 1;
        keys[i] = (int64_t)rows[i] * ncols + (int64_t)cols[i];
    }
    if (bad) { free(keys); free(perm); free(counts); free(cidx64); return -1; }
    orc_sort_indices_i64(keys, nnz, perm);
    for (int64_t i = 0; i < nnz; i++) {
        int64_t p = perm[i];
        col_idx[i] = cols[p];
        cidx64[i] = cols[p];
        csr_vals[i] = vals[p];
        counts[rows[p]] += 1;
    }
    orc_scan_i64(counts, row_ptr, nrows, 0, 0, 0);
    row_ptr[nrows] = nnz;
    orc_spmv_csr_f64(nrows, row_ptr, cidx64, csr_vals, x, y);
    free(keys); free(perm); free(counts); free(cidx64);
    return 0;
}

/* The deterministic triplets of bench/coo_csr_build/coo_csr_build.hyd:18-35:
 * g = i / dup, row = (g*17+3) mod nrows, col = (g*31+7) mod ncols,
 * val = g*13 + i + 1.                                                        */
void orc_coo_csr_bench_inputs(int64_t nrows, int64_t ncols, int64_t nnz, int64_t dup,
                              int64_t* rows, int64_t* cols, int64_t* vals) {
    for (int64_t i = 0; i < nnz; i++) {
        int64_t g = i / dup;
        int64_t r = g * 17 + 3, c = g * 31 + 7;
        rows[i] = r - (r / nrows) * nrows;
        cols[i] = c - (c / ncols) * ncols;
        vals[i] = g * 13 + i + 1;
    }
}
