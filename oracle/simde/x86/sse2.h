/* oracle/simde/x86/sse2.h -- scalar stand-in for the SIMDe SSE2 subset that
 * the reference runtime header includes.  The SIMDe submodule is not vendored
 * with the reference, so this project-written shim lets the unmodified header
 * compile for the oracle's witness build.  Each operation is written from the
 * documented lane semantics of the x86 intrinsic it names (lane-wise IEEE
 * arithmetic, lane 0 = lowest address); nothing here is SIMDe code.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef ORACLE_SIMDE_SSE2_SHIM_H
#define ORACLE_SIMDE_SSE2_SHIM_H
#include <math.h>
#include <string.h>

typedef struct { double v[2]; } simde__m128d;
typedef struct { float v[4]; } simde__m128;

static inline simde__m128d simde_mm_loadu_pd(const double* p) { simde__m128d r; memcpy(r.v, p, sizeof r.v); return r; }
static inline simde__m128d simde_mm_load_pd(const double* p) { return simde_mm_loadu_pd(p); }
static inline void simde_mm_storeu_pd(double* p, simde__m128d a) { memcpy(p, a.v, sizeof a.v); }
static inline void simde_mm_store_pd(double* p, simde__m128d a) { simde_mm_storeu_pd(p, a); }
#define ORC_SHIM_BIN_PD(name, op) \
    static inline simde__m128d name(simde__m128d a, simde__m128d b) { \
        simde__m128d r; r.v[0] = a.v[0] op b.v[0]; r.v[1] = a.v[1] op b.v[1]; return r; }
ORC_SHIM_BIN_PD(simde_mm_add_pd, +)
ORC_SHIM_BIN_PD(simde_mm_sub_pd, -)
ORC_SHIM_BIN_PD(simde_mm_mul_pd, *)
ORC_SHIM_BIN_PD(simde_mm_div_pd, /)
static inline simde__m128d simde_mm_set1_pd(double x) { simde__m128d r; r.v[0] = x; r.v[1] = x; return r; }
static inline simde__m128d simde_mm_setzero_pd(void) { return simde_mm_set1_pd(0.0); }
static inline simde__m128d simde_mm_sqrt_pd(simde__m128d a) { simde__m128d r; r.v[0] = sqrt(a.v[0]); r.v[1] = sqrt(a.v[1]); return r; }
static inline double simde_mm_cvtsd_f64(simde__m128d a) { return a.v[0]; }
/* unpackhi: result = { a[1], b[1] } */
static inline simde__m128d simde_mm_unpackhi_pd(simde__m128d a, simde__m128d b) { simde__m128d r; r.v[0] = a.v[1]; r.v[1] = b.v[1]; return r; }

static inline simde__m128 simde_mm_loadu_ps(const float* p) { simde__m128 r; memcpy(r.v, p, sizeof r.v); return r; }
static inline simde__m128 simde_mm_load_ps(const float* p) { return simde_mm_loadu_ps(p); }
static inline void simde_mm_storeu_ps(float* p, simde__m128 a) { memcpy(p, a.v, sizeof a.v); }
static inline void simde_mm_store_ps(float* p, simde__m128 a) { simde_mm_storeu_ps(p, a); }
#define ORC_SHIM_BIN_PS(name, op) \
    static inline simde__m128 name(simde__m128 a, simde__m128 b) { \
        simde__m128 r; for (int i = 0; i < 4; i++) r.v[i] = a.v[i] op b.v[i]; return r; }
ORC_SHIM_BIN_PS(simde_mm_add_ps, +)
ORC_SHIM_BIN_PS(simde_mm_sub_ps, -)
ORC_SHIM_BIN_PS(simde_mm_mul_ps, *)
ORC_SHIM_BIN_PS(simde_mm_div_ps, /)
static inline simde__m128 simde_mm_set1_ps(float x) { simde__m128 r; for (int i = 0; i < 4; i++) r.v[i] = x; return r; }
static inline simde__m128 simde_mm_setzero_ps(void) { return simde_mm_set1_ps(0.0f); }
#endif
