/*
 * hpss_oracle.h -- CPU restatement of the semblance hot path of
 * HighPerformanceSeismicStacking, used ONLY to check against (tests, smoke(),
 * and the CPU-baseline leg of bench.py).  It is test infrastructure: no
 * product code path links, loads or calls it.
 *
 * Every function restates a reference kernel or driver step in plain C, in
 * IEEE arithmetic (no fast-math), once with float and once with double
 * (suffix _f32 / _f64).  The float instantiation follows the reference's FP32
 * operation order; the double one is the FP64 oracle the results are judged
 * against.
 *
 * Parity pins: the reference ships no tests, fixtures or data.  The oracle is
 * pinned against (1) outputs of the reference's own CUDA kernels compiled from
 * the reference sources and run on a GB300 (fixtures under tests/golden/, made
 * by tests/golden/make_reference_golden.py) and (2) analytic known-answer
 * cases (tests/test_oracle.py).
 */
#ifndef HPSS_ORACLE_H
#define HPSS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_CMP = 0, ORACLE_ZOCRS = 1, ORACLE_OCT = 2 };

/* Linear-search evaluation for ONE midpoint m0.
 *   samples   [*][stride] row-major trace amplitudes (whole line)
 *   sel       indices (into the whole line) of the traces used for m0
 *   params    AoS [P][np] candidate parameters exactly as the reference's
 *             parameter array stores them: CMP {4/v^2}, ZOCRS {4/v^2, A, B},
 *             OCT {4/v^2, slope}
 *   sembl, stack [S][P]: per (t0 sample, candidate) semblance and stack
 *   not_used  optional [S][P] (OCT): traces skipped for a displaced midpoint
 * Follows cuda/src/semblance/kernel/{cmp,zocrs,oct}/linear_search.cu
 * (computeSemblancesFor*) and common/include/gpu/interface.h:20-55. */
void oracle_ls_eval_f32(int model, const float *samples, uint32_t stride,
                        uint32_t S, float dt, int tau,
                        const float *mid, const float *hoff,
                        const uint32_t *sel, uint32_t nsel, float m0,
                        float apm, float h0, const float *params, uint32_t P,
                        float *sembl, float *stack, float *not_used,
                        int nthreads);
void oracle_ls_eval_f64(int model, const float *samples, uint32_t stride,
                        uint32_t S, float dt, int tau,
                        const float *mid, const float *hoff,
                        const uint32_t *sel, uint32_t nsel, float m0,
                        float apm, float h0, const float *params, uint32_t P,
                        double *sembl, double *stack, double *not_used,
                        int nthreads);

/* The same evaluation on the t0 samples sidx[0..nS) only (all candidates):
 * tables [nS][P]. */
void oracle_ls_eval_samples_f32(int model, const float *samples,
                                uint32_t stride, uint32_t S, float dt, int tau,
                                const float *mid, const float *hoff,
                                const uint32_t *sel, uint32_t nsel, float m0,
                                float apm, float h0, const float *params,
                                uint32_t P, const uint32_t *sidx, uint32_t nS,
                                float *sembl, float *stack, int nthreads);
void oracle_ls_eval_samples_f64(int model, const float *samples,
                                uint32_t stride, uint32_t S, float dt, int tau,
                                const float *mid, const float *hoff,
                                const uint32_t *sel, uint32_t nsel, float m0,
                                float apm, float h0, const float *params,
                                uint32_t P, const uint32_t *sidx, uint32_t nS,
                                double *sembl, double *stack, int nthreads);

/* Argmax over candidates with the reference's strict '>' scan from -1
 * (lowest index wins ties; NaN never wins).  best_idx[s] = -1 if none.
 * Follows selectBestSemblancesFor* (cuda/src/semblance/kernel/cmp/
 * linear_search.cu:83-115 and the zocrs/oct twins). */
void oracle_argmax_f32(const float *sembl, uint32_t S, uint32_t P,
                       int32_t *best_idx);
void oracle_argmax_f64(const double *sembl, uint32_t S, uint32_t P,
                       int32_t *best_idx);

/* Parameter grid, as buildParameterArrayFor* (cmp/linear_search.cu:4-17,
 * zocrs/linear_search.cu:4-34, oct/linear_search.cu:4-28) with the steps of
 * LinearSearchAlgorithm::setupDiscretizationSteps (LinearSearchAlgorithm.cpp
 * :129-141).  First parameter slowest, last fastest.  Writes np*P floats. */
void oracle_build_grid(int model, const float *lower, const float *upper,
                       const uint32_t *gran, float *params);

/* Inclusive grid: both bounds included, velocity uniform in 4/v^2 (the
 * engine's HPSS_GRID_INCLUSIVE; no reference counterpart). */
void oracle_build_grid_inclusive(int model, const float *lower, const float *upper,
                                 const uint32_t *gran, float *params);

/* Trace selection masks (mask[i] for every trace of the line).
 * CMP:   m == m0 (cmp/common.cu:3-15)
 * ZOCRS: |m0 - m| <= apm (zocrs/common.cu:3-16)
 * OCT:   any (t0 sample, candidate) of `cands` ([n][2] = {4/v^2, slope})
 *        gives a valid displaced midpoint with |m - mh| <= apm
 *        (oct/linear_search.cu:155-192). */
void oracle_select(int model, const float *mid, const float *hoff,
                   uint32_t ntr, float m0, float apm, float h0, uint32_t S,
                   float dt, const float *cands, uint32_t ncand,
                   uint8_t *mask);

/* Stretch-free evaluation for one m0: candidates n in [-nmax, nmax]; the
 * model parameters for every sample come from a prior result, SoA
 * [np][S] with RAW velocity first (cmp/stretch_free.cu:4-66,
 * zocrs/stretch_free.cu:4-85, oct/stretch_free.cu:5-97).  sembl/stack
 * are [S][2*nmax+1]. */
void oracle_sf_eval_f32(int model, const float *samples, uint32_t stride,
                        uint32_t S, float dt, int tau, const float *mid,
                        const float *hoff, const uint32_t *sel, uint32_t nsel,
                        float m0, float apm, float h0, const float *prior,
                        int nmax, float *sembl, float *stack, float *not_used,
                        int nthreads);
void oracle_sf_eval_f64(int model, const float *samples, uint32_t stride,
                        uint32_t S, float dt, int tau, const float *mid,
                        const float *hoff, const uint32_t *sel, uint32_t nsel,
                        float m0, float apm, float h0, const float *prior,
                        int nmax, double *sembl, double *stack,
                        double *not_used, int nthreads);

/* Semblance of explicit per-sample candidate sets (used to score the
 * differential-evolution results): cands AoS [S][n][np] in RAW parameters
 * (velocity, not 4/v^2), as the reference's DE population
 * (cmp/differential_evolution.cu:4-65 and twins). */
void oracle_eval_raw_f64(int model, const float *samples, uint32_t stride,
                         uint32_t S, float dt, int tau, const float *mid,
                         const float *hoff, const uint32_t *sel,
                         uint32_t nsel, float m0, float apm, float h0,
                         const float *cands, uint32_t n, double *sembl,
                         double *stack, int nthreads);
void oracle_eval_raw_f32(int model, const float *samples, uint32_t stride,
                         uint32_t S, float dt, int tau, const float *mid,
                         const float *hoff, const uint32_t *sel,
                         uint32_t nsel, float m0, float apm, float h0,
                         const float *cands, uint32_t n, float *sembl,
                         float *stack, int nthreads);

int oracle_max_threads(void);

/* Differential evolution: the engine's counter-based random stream
 * (Philox-4x32-10 keyed by the seed) and the initial population drawn from
 * it; per-sample OCT selection with raw (velocity, slope) candidates. */
void oracle_de_uniforms(uint64_t seed, uint32_t m0i, uint32_t s, uint32_t ind,
                        uint32_t gen, uint32_t n, float *out);
void oracle_de_initial_population(uint64_t seed, uint32_t m0i, uint32_t S,
                                  uint32_t pop, int np, const float *lo,
                                  const float *hi, float *out);
void oracle_select_oct_per_sample(const float *mid, const float *hoff,
                                  uint32_t ntr, float m0, float apm, float h0,
                                  uint32_t S, float dt, const float *cands,
                                  uint32_t n, uint8_t *mask);

#ifdef __cplusplus
}
#endif
#endif
