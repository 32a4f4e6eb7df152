/*
 * hpss_oracle.c -- CPU restatement of the reference's semblance hot path.
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker; never by the product path.
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
