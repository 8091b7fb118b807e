/* oracle/simde/x86/avx.h -- scalar stand-in for the SIMDe AVX subset that the
 * reference runtime header includes (see sse2.h in this directory).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef ORACLE_SIMDE_AVX_SHIM_H
#define ORACLE_SIMDE_AVX_SHIM_H
#include "sse2.h"

typedef struct { double v[4]; } simde__m256d;

static inline simde__m256d simde_mm256_loadu_pd(const double* p) { simde__m256d r; memcpy(r.v, p, sizeof r.v); return r; }
static inline void simde_mm256_storeu_pd(double* p, simde__m256d a) { memcpy(p, a.v, sizeof a.v); }
#define ORC_SHIM_BIN_PD4(name, op) \
    static inline simde__m256d name(simde__m256d a, simde__m256d b) { \
        simde__m256d r; for (int i = 0; i < 4; i++) r.v[i] = a.v[i] op b.v[i]; return r; }
ORC_SHIM_BIN_PD4(simde_mm256_add_pd, +)
ORC_SHIM_BIN_PD4(simde_mm256_sub_pd, -)
ORC_SHIM_BIN_PD4(simde_mm256_mul_pd, *)
ORC_SHIM_BIN_PD4(simde_mm256_div_pd, /)
static inline simde__m256d simde_mm256_set1_pd(double x) { simde__m256d r; for (int i = 0; i < 4; i++) r.v[i] = x; return r; }
static inline simde__m256d simde_mm256_setzero_pd(void) { return simde_mm256_set1_pd(0.0); }
static inline simde__m256d simde_mm256_sqrt_pd(simde__m256d a) { simde__m256d r; for (int i = 0; i < 4; i++) r.v[i] = sqrt(a.v[i]); return r; }
/* extractf128: imm 0 -> lanes {0,1}, imm 1 -> lanes {2,3} */
static inline simde__m128d simde_mm256_extractf128_pd(simde__m256d a, int imm) {
    simde__m128d r; r.v[0] = a.v[(imm & 1) * 2]; r.v[1] = a.v[(imm & 1) * 2 + 1]; return r; }
#endif
