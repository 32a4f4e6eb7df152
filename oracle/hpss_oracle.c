/*
 * hpss_oracle.c -- CPU restatement of the reference's semblance hot path.
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py to check against; never by the product path.
 *
 * Built with -O2 -ffp-contract=off so that x86-64 and aarch64 hosts produce
 * identical float results (no fused multiply-add contraction).
 */
#include "hpss_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXW 64

/* gpu_error_code (common/include/gpu/interface.h:12-18) */
enum { OERR_NONE = 0, OERR_DIV_ZERO = 1, OERR_NEG_SQRT = 2 };

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Float -> int truncation with the GPU's saturating convert semantics
 * (cvt.rzi.s32.f32: NaN -> 0, out of range -> INT_MIN / INT_MAX), so the
 * oracle is defined where C's (int) cast is not. */
static inline int64_t f2i_rz(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return 2147483647;
    if (x <= -2147483648.0) return -2147483648LL;
    return (int64_t)x;
}

#define REAL float
#define SUFFIX _f32
#define SQRT sqrtf
#define FABS fabsf
#include "hpss_oracle_impl.inc"
#undef REAL
#undef SUFFIX
#undef SQRT
#undef FABS

#define REAL double
#define SUFFIX _f64
#define SQRT sqrt
#define FABS fabs
#include "hpss_oracle_impl.inc"
#undef REAL
#undef SUFFIX
#undef SQRT
#undef FABS

/* buildParameterArrayFor* + setupDiscretizationSteps: step_j = (U-L)/G in
 * float; value = L + idx*step; velocity stored as 4/v^2. */
void oracle_build_grid(int model, const float *lower, const float *upper,
                       const uint32_t *gran, float *params) {
    int np = model == ORACLE_CMP ? 1 : (model == ORACLE_ZOCRS ? 3 : 2);
    float step[3];
    uint32_t total = 1;
    for (int j = 0; j < np; j++) {
        step[j] = (upper[j] - lower[j]) / (float)gran[j];
        total *= gran[j];
    }
    for (uint32_t i = 0; i < total; i++) {
        uint32_t rem = i;
        uint32_t idx[3] = {0, 0, 0};
        for (int j = np - 1; j >= 0; j--) {
            idx[j] = rem % gran[j];
            rem /= gran[j];
        }
        for (int j = 0; j < np; j++) {
            /* the reference's device code contracts min + idx*inc into one
             * fused multiply-add (single rounding) */
            float v = fmaf((float)idx[j], step[j], lower[j]);
            params[(size_t)i * np + j] = j == 0 ? 4.0f / (v * v) : v;
        }
    }
}

/* Inclusive grid (the engine's HPSS_GRID_INCLUSIVE): both bounds included,
 * velocity uniform in c = 4/v^2 from 4/L^2 down to 4/U^2, the others uniform
 * from L to U; value = fmaf(idx, step, first), the last index takes the end
 * value exactly.  Same order as oracle_build_grid. */
void oracle_build_grid_inclusive(int model, const float *lower, const float *upper,
                                 const uint32_t *gran, float *params) {
    int np = model == ORACLE_CMP ? 1 : (model == ORACLE_ZOCRS ? 3 : 2);
    float first[3], last[3], step[3];
    uint32_t total = 1;
    for (int j = 0; j < np; j++) {
        first[j] = j == 0 ? 4.0f / (lower[0] * lower[0]) : lower[j];
        last[j] = j == 0 ? 4.0f / (upper[0] * upper[0]) : upper[j];
        step[j] = gran[j] > 1 ? (last[j] - first[j]) / (float)(gran[j] - 1) : 0.0f;
        total *= gran[j];
    }
    for (uint32_t i = 0; i < total; i++) {
        uint32_t rem = i;
        uint32_t idx[3] = {0, 0, 0};
        for (int j = np - 1; j >= 0; j--) {
            idx[j] = rem % gran[j];
            rem /= gran[j];
        }
        for (int j = 0; j < np; j++) {
            float v = (gran[j] > 1 && idx[j] == gran[j] - 1)
                          ? last[j]
                          : fmaf((float)idx[j], step[j], first[j]);
            params[(size_t)i * np + j] = v;
        }
    }
}

void oracle_select(int model, const float *mid, const float *hoff,
                   uint32_t ntr, float m0, float apm, float h0, uint32_t S,
                   float dt, const float *cands, uint32_t ncand,
                   uint8_t *mask) {
    for (uint32_t i = 0; i < ntr; i++) {
        if (model == ORACLE_CMP) {
            mask[i] = (m0 == mid[i]);
        } else if (model == ORACLE_ZOCRS) {
            mask[i] = fabsf(m0 - mid[i]) <= apm;
        } else {
            float m = mid[i], h = hoff[i], mh;
            uint8_t used = 0;
            for (uint32_t s = 0; !used && s < S; s++) {
                float t0 = (float)s * dt;
                for (uint32_t p = 0; !used && p < ncand; p++) {
                    float c = cands[2 * p], slope = cands[2 * p + 1];
                    int e = oct_mh_f32(h, h0, t0, m0, c, slope, &mh);
                    used = (e == OERR_NONE && fabsf(m - mh) <= apm);
                }
            }
            mask[i] = used;
        }
    }
}

/* ---- differential evolution helpers (engine's random stream) ----------
 * Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), as the engine keys it:
 * key = seed (lo, hi words); counter = (gen << 8 | draw block, individual,
 * sample, midpoint key: the midpoint's FP32 bit pattern).  Uniforms in (0, 1]:
 * ((v >> 8) + 1) * 2^-24. */
static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

static float u01(uint32_t v) { return (float)((v >> 8) + 1u) * (1.0f / 16777216.0f); }

/* First n uniforms of the stream of (midpoint key, sample, individual,
 * generation). */
void oracle_de_uniforms(uint64_t seed, uint32_t m0i, uint32_t s, uint32_t ind,
                        uint32_t gen, uint32_t n, float *out) {
    uint32_t ctr = gen << 8;
    for (uint32_t i = 0; i < n; i += 4) {
        uint32_t c[4] = {ctr++, ind, s, m0i};
        philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        for (uint32_t j = 0; j < 4 && i + j < n; j++) out[i + j] = u01(c[j]);
    }
}

/* Initial population [S][pop][np]: x_j = lo_j + U * (hi_j - lo_j)
 * (startPopulations, common/differential_evolution.cu:19-41). */
void oracle_de_initial_population(uint64_t seed, uint32_t m0i, uint32_t S,
                                  uint32_t pop, int np, const float *lo,
                                  const float *hi, float *out) {
    float u[4];
    for (uint32_t s = 0; s < S; s++)
        for (uint32_t i = 0; i < pop; i++) {
            oracle_de_uniforms(seed, m0i, s, i, 0, (uint32_t)np, u);
            for (int j = 0; j < np; j++)
                out[((size_t)s * pop + i) * np + j] = fmaf(u[j], hi[j] - lo[j], lo[j]);
        }
}

/* OCT selection with per-sample raw candidates cands [S][n][2] (velocity,
 * slope), c = 4/v^2 (oct/differential_evolution.cu:130-168). */
void oracle_select_oct_per_sample(const float *mid, const float *hoff,
                                  uint32_t ntr, float m0, float apm, float h0,
                                  uint32_t S, float dt, const float *cands,
                                  uint32_t n, uint8_t *mask) {
    for (uint32_t i = 0; i < ntr; i++) {
        float m = mid[i], h = hoff[i], mh;
        uint8_t used = 0;
        for (uint32_t s = 0; !used && s < S; s++) {
            float t0 = (float)s * dt;
            for (uint32_t p = 0; !used && p < n; p++) {
                const float *cd = cands + ((size_t)s * n + p) * 2;
                float v = cd[0];
                float c = 4.0f / (v * v);
                int e = oct_mh_f32(h, h0, t0, m0, c, cd[1], &mh);
                used = (e == OERR_NONE && fabsf(m - mh) <= apm);
            }
        }
        mask[i] = used;
    }
}
