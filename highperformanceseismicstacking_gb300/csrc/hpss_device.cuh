// hpss_device.cuh -- device-side building blocks shared by the semblance
// kernels: the three traveltime models and the semblance window.
//
// The arithmetic restates, operation for operation, the reference's
// COMPUTE_SEMBLANCE / REDUCE_SEMBLANCE_STACK macros
// (common/include/gpu/interface.h:26-55) and the OCT helpers
// computeDisplacedMidpoint / computeTime
// (cuda/include/semblance/kernel/oct/common.cuh:7-94).  The library is built
// with --use_fast_math like the reference (cuda/Makefile:26), so that with the
// same operation order the same instructions are generated and the window
// index and selected grid index come out bit-identical.
#pragma once

#include <cuda_fp16.h>

#include <cstdint>

#include "hpss_internal.h"

namespace hpss {

// gpu_error_code (common/include/gpu/interface.h:12-18).
enum DevErr : int { DE_OK = 0, DE_DIV_ZERO = 1, DE_NEG_SQRT = 2 };

// The traveltime expressions are written with explicit round-to-nearest
// intrinsics (__fmaf_rn / __fmul_rn / __fadd_rn are never re-fused by the
// compiler), so every kernel of this library computes them with one fixed
// sequence of roundings.  The sequence is the one the reference's compiled
// kernels use (nvcc contracts a*b + c*d into one fused multiply-add, keeping
// the product of loop-invariant factors separate); verified bit for bit
// against the reference kernels' outputs (tests/golden).

// CMP: t = sqrt(t0^2 + c h^2), c = 4/v^2 (cmp/linear_search.cu:57).
__device__ __forceinline__ float cmp_time(float t0, float c, float h_sq) {
    return sqrtf(__fmaf_rn(c, h_sq, __fmul_rn(t0, t0)));
}

// ZO-CRS squared time (t0 + A dm)^2 + B dm^2 + C h^2
// (zocrs/linear_search.cu:83-87).
__device__ __forceinline__ float zocrs_t2(float t0, float c, float a, float b,
                                          float dm, float h_sq) {
    const float x = __fmaf_rn(a, dm, t0);
    const float y = __fmaf_rn(__fmul_rn(b, dm), dm, __fmul_rn(x, x));
    return __fmaf_rn(c, h_sq, y);
}

// ZO-CRS time; false when the squared time is negative (window skipped).
__device__ __forceinline__ bool zocrs_time(float t0, float c, float a, float b,
                                           float dm, float h_sq, float *t) {
    const float tmp = zocrs_t2(t0, c, a, b, dm, h_sq);
    if (tmp >= 0) {
        *t = sqrtf(tmp);
        return true;
    }
    return false;
}

// ZO-CRS time with the squared time (t0 + A dm)^2 + B dm^2 + C h^2 formed in
// FP64 from the FP32 inputs (h^2 as the FP32 product the reference's host
// code forms) and the time rounded to FP32 once; false when the square is
// negative (window skipped).  The precision mode HPSS_PREC_FP64_TRAVELTIME.
__device__ __forceinline__ bool zocrs_time_tt64(float t0, float c, float a, float b, float dm,
                                                float h_sq, float *t) {
    const double x = (double)t0 + (double)a * (double)dm;
    const double tmp = x * x + (double)b * (double)dm * (double)dm + (double)c * (double)h_sq;
    *t = tmp >= 0 ? (float)sqrt(tmp) : 0.f;
    return tmp >= 0;
}

// OCT displaced midpoint and time in FP64 (same formulas and operation
// order as oct/common.cuh:7-94) from the FP32 inputs; returns as model_time
// (-1 not used: displaced-midpoint error or |m - mh| > apm; 0 window skipped:
// time error; 1 time valid).
__device__ __forceinline__ int oct_time_d(double t0, double c, double slope, double m, double h,
                                          double m0, double apm, double h0, double *t) {
    const double theta = t0 * slope;
    const double gamma = 2 * sqrt(h * h + h0 * h0);
    const double tn0_sq = t0 * t0 - c * h0 * h0;
    const double theta_sq = theta * theta, gamma_sq = gamma * gamma, tn0_quad = tn0_sq * tn0_sq;
    double arg = tn0_quad * tn0_quad + tn0_quad * theta_sq * gamma_sq +
                 16 * h * h * h0 * h0 * theta_sq * theta_sq;
    if (arg < 0) return -1;
    arg = theta_sq * gamma_sq + 2 * tn0_quad + 2 * sqrt(arg);
    if (arg == 0) return -1;
    const double mh = m0 + 2 * theta * (h * h - h0 * h0) / sqrt(arg);
    if (fabs(m - mh) > apm) return -1;
    const double w1 = (h + h0) * (h + h0) - (mh - m0) * (mh - m0);
    const double w2 = (h - h0) * (h - h0) - (mh - m0) * (mh - m0);
    if (w1 < 0 || w2 < 0) return 0;
    const double u = sqrt(w1) + sqrt(w2);
    double th = t0;
    if (fabs(h) > fabs(h0)) {
        if (!u) return 0;
        const double sa = c * h * h + 4 * h * h / (u * u) * tn0_sq;
        if (sa < 0) return 0;
        th = sqrt(sa);
    } else if (fabs(h) < fabs(h0)) {
        if (!h0) return 0;
        const double sa = c * h * h + u * u / (4 * h0 * h0) * tn0_sq;
        if (sa < 0) return 0;
        th = sqrt(sa);
    }
    const double tn_sq = th * th - c * h * h;
    if (!th || !tn0_sq) return 0;
    const double ah = (t0 * tn_sq) / (th * tn0_sq) * slope;
    *t = th + ah * (m - mh);
    return 1;
}

// The same with the time rounded to FP32 once (precision mode
// HPSS_PREC_FP64_TRAVELTIME).
__device__ __forceinline__ int oct_time_f64(float t0, float c, float slope, float m, float h,
                                            float m0, float apm, float h0, float *t) {
    double td = 0;
    const int ok = oct_time_d(t0, c, slope, m, h, m0, apm, h0, &td);
    if (ok > 0) *t = (float)td;
    return ok;
}

// Knuth's two-sum: s + x as sum and rounding error, branch-free; the
// error is kept in a compensation term (compensated summation of the window
// sums, precision mode HPSS_PREC_COMPENSATED).
__device__ __forceinline__ void two_sum_acc(float &s, float &comp, float x) {
    const float t = __fadd_rn(s, x);
    const float z = __fsub_rn(t, s);
    comp = __fadd_rn(comp, __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(x, z)));
    s = t;
}

// t0^2 - c h0^2 of the OCT formulas.
__device__ __forceinline__ float oct_tn0_sq(float t0, float c, float h0) {
    return __fmaf_rn(t0, t0, -__fmul_rn(__fmul_rn(c, h0), h0));
}

// The OCT formulas factored by what their terms depend on, each factor
// rounded exactly as in the one-expression form: per trace (h, h0) and per
// (t0, candidate).  Kernels that visit many traces per candidate take the
// trace factors from a table (oct_trace_table_kernel) and the candidate
// factors out of the trace loop; the values are the same bit for bit.
struct OctCand {
    float ts;        // theta^2, theta = t0 * slope
    float tn0_sq;    // t0^2 - c h0^2
    float tq;        // tn0_sq^2
    float tqts;      // tq * theta^2
    float twoTq;     // 2 tq
    float twoTheta;  // 2 theta
};
__device__ __forceinline__ OctCand oct_cand(float t0, float c, float slope, float h0) {
    OctCand k;
    const float theta = __fmul_rn(t0, slope);
    k.ts = __fmul_rn(theta, theta);
    k.tn0_sq = oct_tn0_sq(t0, c, h0);
    k.tq = __fmul_rn(k.tn0_sq, k.tn0_sq);
    k.tqts = __fmul_rn(k.tq, k.ts);
    k.twoTq = __fmul_rn(2.f, k.tq);
    k.twoTheta = 2.f * theta;
    return k;
}

// Trace factors of the displaced midpoint: gamma^2 = (2 sqrt(h^2 + h0^2))^2,
// 16 h^2 h0^2 and h^2 - h0^2 (the product h*h is rounded on its own and the
// h0 product is fused -- fractional half-offsets tell the forms apart).
struct OctTrace {
    float gs, p16h, dif;
};
__device__ __forceinline__ OctTrace oct_trace(float h, float h0) {
    OctTrace f;
    const float hh = __fmul_rn(h, h);
    const float gamma = 2 * sqrtf(__fmaf_rn(h0, h0, hh));
    f.gs = __fmul_rn(gamma, gamma);
    f.p16h = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(16.f, h), h), h0), h0);
    f.dif = __fmaf_rn(-h0, h0, hh);
    return f;
}

// OCT displaced midpoint (oct/common.cuh:7-35) from its factors.
__device__ __forceinline__ int oct_mh(const OctCand &k, float gs, float p16h, float dif,
                                      float m0, float *mh) {
    // tq^2 + tq ts gs + 16 h^2 h0^2 ts^2 as the reference's OCT kernel rounds
    // it: tq ts gs as products, tq^2 fused onto them, the last product fused;
    // then ts gs + 2 tq as a plain add (matched against every entry of the
    // reference kernel's semblance tables on the OCT fixtures)
    float arg = __fmaf_rn(k.tq, k.tq, __fmul_rn(k.tqts, gs));
    arg = __fmaf_rn(__fmul_rn(p16h, k.ts), k.ts, arg);
    if (arg < 0) return DE_NEG_SQRT;
    arg = __fadd_rn(__fadd_rn(__fmul_rn(k.ts, gs), k.twoTq), __fmul_rn(2.f, sqrtf(arg)));
    if (arg == 0) return DE_DIV_ZERO;
    // m0 + 2 theta (h^2 - h0^2) / sqrt(.): the reference's fast-math build
    // divides by multiplying with the approximate reciprocal and fuses that
    // product with the add of m0 -- fma(2 theta dif, rcp(sqrt(.)), m0)
    *mh = __fmaf_rn(__fmul_rn(k.twoTheta, dif), __fdividef(1.0f, sqrtf(arg)), m0);
    return DE_OK;
}

// oct_mh without the early returns: every operation is carried out whatever
// the error (the codes are the same, and so is *mh when the code is DE_OK),
// so that a thread can run several of these chains side by side.
__device__ __forceinline__ int oct_mh_all(const OctCand &k, float gs, float p16h, float dif,
                                          float m0, float *mh) {
    float arg = __fmaf_rn(k.tq, k.tq, __fmul_rn(k.tqts, gs));
    arg = __fmaf_rn(__fmul_rn(p16h, k.ts), k.ts, arg);
    const float arg2 =
        __fadd_rn(__fadd_rn(__fmul_rn(k.ts, gs), k.twoTq), __fmul_rn(2.f, sqrtf(arg)));
    *mh = __fmaf_rn(__fmul_rn(k.twoTheta, dif), __fdividef(1.0f, sqrtf(arg2)), m0);
    return arg < 0 ? DE_NEG_SQRT : (arg2 == 0 ? DE_DIV_ZERO : DE_OK);
}

// OCT displaced midpoint (oct/common.cuh:7-35).
__device__ __forceinline__ int oct_displaced_midpoint(float h, float h0,
                                                      float t0, float m0,
                                                      float c, float slope,
                                                      float *mh) {
    const OctTrace f = oct_trace(h, h0);
    return oct_mh(oct_cand(t0, c, slope, h0), f.gs, f.p16h, f.dif, m0, mh);
}

// OCT traveltime at the displaced midpoint (oct/common.cuh:37-94), with
// tn0_sq = t0^2 - c h0^2 given.
__device__ __forceinline__ int oct_time_k(float h, float h0, float t0, float tn0_sq, float m0,
                                          float m, float mh, float c, float slope,
                                          float *out) {
    const float b = __fsub_rn(mh, m0);
    const float bb = __fmul_rn(b, b);
    const float ap = __fadd_rn(h, h0), am = __fsub_rn(h, h0);
    const float w1 = __fmaf_rn(ap, ap, -bb);
    const float w2 = __fmaf_rn(am, am, -bb);
    if (w1 < 0 || w2 < 0) return DE_NEG_SQRT;
    const float u = __fadd_rn(sqrtf(w1), sqrtf(w2));
    float th = t0;
    if (fabsf(h) > fabsf(h0)) {
        if (!u) return DE_DIV_ZERO;
        const float q = __fmul_rn(__fmul_rn(4.f, h), h) / __fmul_rn(u, u);
        const float arg = __fmaf_rn(__fmul_rn(c, h), h, __fmul_rn(q, tn0_sq));
        if (arg < 0) return DE_NEG_SQRT;
        th = sqrtf(arg);
    } else if (fabsf(h) < fabsf(h0)) {
        if (!h0) return DE_DIV_ZERO;
        const float q = __fmul_rn(u, u) / __fmul_rn(__fmul_rn(4.f, h0), h0);
        const float arg = __fmaf_rn(__fmul_rn(c, h), h, __fmul_rn(q, tn0_sq));
        if (arg < 0) return DE_NEG_SQRT;
        th = sqrtf(arg);
    }
    const float tn_sq = __fmaf_rn(th, th, -__fmul_rn(__fmul_rn(c, h), h));
    if (!th || !tn0_sq) return DE_DIV_ZERO;
    const float ah = __fmul_rn(__fmul_rn(t0, tn_sq) / __fmul_rn(th, tn0_sq), slope);
    *out = __fmaf_rn(ah, __fsub_rn(m, mh), th);
    return DE_OK;
}

// OCT traveltime of one trace for the candidate factors k (candidate c,
// slope), trace factors f and midpoint m, half-offset h; returns as
// model_time below.
__device__ __forceinline__ int oct_model_time(const OctCand &k, float gs, float p16h, float dif,
                                              float t0, float c, float slope, float m, float h,
                                              float m0, float apm, float h0, float *t) {
    float mh;
    int e = oct_mh(k, gs, p16h, dif, m0, &mh);
    if (e != DE_OK || fabsf(m - mh) > apm) return -1;
    e = oct_time_k(h, h0, t0, k.tn0_sq, m0, m, mh, c, slope, t);
    return e == DE_OK ? 1 : 0;
}

// Traveltime of one trace for one candidate, dispatching on the model.
// Returns: 1 = time valid, 0 = window skipped (ZO-CRS negative square,
// OCT computeTime error), -1 = trace not used (OCT displaced midpoint error
// or |m - mh| > apm; counted in notUsed).  The candidate is (c = 4/v^2,
// p1, p2) as stored in the reference's parameter arrays.
template <int MODEL>
__device__ __forceinline__ int model_time(float t0, float c, float p1,
                                          float p2, float m, float h,
                                          float h_sq, float m0, float apm,
                                          float h0, float *t) {
    if (MODEL == kModelCmp) {
        *t = cmp_time(t0, c, h_sq);
        return 1;
    } else if (MODEL == kModelZocrs) {
        float dm = m - m0;
        return zocrs_time(t0, c, p1, p2, dm, h_sq, t) ? 1 : 0;
    } else {
        const OctTrace f = oct_trace(h, h0);
        return oct_model_time(oct_cand(t0, c, p1, h0), f.gs, f.p16h, f.dif, t0, c, p1, m, h, m0,
                              apm, h0, t);
    }
}

// Window index of a traveltime: tIndex = t / dt, k = (int)tIndex,
// frac = tIndex - k (interface.h:27-29).  The window is used iff
// k - tau >= 0 && k + tau + 1 < S (interface.h:30).
struct WinIdx {
    int k;
    float frac;
};
__device__ __forceinline__ WinIdx window_index(float t, float dt) {
    float tIndex = t / dt;
    WinIdx w;
    w.k = (int)tIndex;
    w.frac = tIndex - (float)w.k;
    return w;
}
__device__ __forceinline__ bool window_in_trace(int k, int tau, int S) {
    return (k - tau >= 0) && (k + tau + 1 < S);
}

// REDUCE_SEMBLANCE_STACK (interface.h:46-55).
__device__ __forceinline__ void reduce_semblance(const float *num, float lin,
                                                 float den, int w,
                                                 unsigned used, float *sembl,
                                                 float *stack) {
    float s = 0, k = 0;
    if (used > 0) {
        float sn = 0;
        for (int j = 0; j < w; j++) sn += num[j] * num[j];
        s = sn / (used * den);
        k = lin / (used * w);
    }
    *sembl = s;
    *stack = k;
}

// Argmax combine with the reference's scan semantics: higher semblance wins,
// equal semblance -> lower candidate index wins (strict '>' scanning upwards
// from -1, cmp/linear_search.cu:98-110).  NaN never enters (strict '>').
struct Best {
    float sembl;
    float stack;
    uint32_t p;
};
__device__ __forceinline__ bool better(float s1, uint32_t p1, float s0,
                                       uint32_t p0) {
    return s1 > s0 || (s1 == s0 && p1 < p0);
}

// Runner-up tracking for the near-tie count: `second` is the largest
// semblance of the candidates other than the chosen one (-1: none).  A sample
// is a near-tie when its best semblance is positive and the runner-up lies
// within kNearTieRel * max(best, 1e-3) of it -- where another rounding order
// could choose another candidate.  NaN semblances never enter.
__device__ __forceinline__ void top2_offer(float s, float best, float &second) {
    // called before `best` is updated with s
    if (s > best) second = best;
    else if (s > second) second = s;
}
__device__ __forceinline__ void top2_merge(float b2, uint32_t p2, float s2, float &b1,
                                           uint32_t &p1, float &s1) {
    if (better(b2, p2, b1, p1)) {
        s1 = fmaxf(b1, s2);
        b1 = b2;
        p1 = p2;
    } else {
        s1 = fmaxf(s1, b2);
    }
}
__device__ __forceinline__ bool near_tie(float best, float second) {
    return best > 0.f && second >= 0.f && best - second <= kNearTieRel * fmaxf(best, 1e-3f);
}

// Displaced-midpoint test for a box of (t0, slope) at once, h0 = 0.  There
// the OCT formula (oct/common.cuh:7-35) reduces to
//     mh - m0 = 2 s h^2 / (t0 + sqrt(t0^2 + 4 s^2 h^2))
// (sqrt(arg2) = t0 (t0 + sqrt(t0^2 + 4 s^2 h^2)) in real arithmetic), which
// increases with the slope s and, for a fixed s, moves toward 0 as t0 grows.
// So over t0 in [t0Lo, t0Hi] and s in [sLo, sHi] mh lies between its values
// at two corners, and a trace whose midpoint is farther than apm from that
// whole interval fails the per-(t0, candidate) test of every member of the
// box: a warp counts it as not used without evaluating it lane by lane.  The
// margin covers the FP32 roundings of both forms (relative 1e-4 of the
// displacement, 1e-5 of the coordinates; the two FP32 evaluations differ
// from the real value by a few ulps).  The exact per-lane test still decides
// every trace the box keeps, so results and not-used counts are those of the
// per-lane test.  Used with t0Lo >= kOctBoxMinT0 (the FP32 terms of the
// reference's form stay normal there); t0 = 0 fails the exact test anyway
// (division by zero) and stays out of the box.  tf = {m, gamma^2 (= 4 h^2),
// 16 h^2 h0^2, h^2 - h0^2 (= h^2)} from the line's factor table.
constexpr float kOctBoxMinT0 = 1e-4f;
__device__ __forceinline__ bool oct_box_may_pass(const float4 &tf, float sLo, float sHi,
                                                 float t0Lo, float t0Hi, float m0, float apm) {
    const float tForHi = sHi > 0.f ? t0Lo : t0Hi;
    const float tForLo = sLo > 0.f ? t0Hi : t0Lo;
    const float hi = 2.f * sHi * tf.w / (tForHi + sqrtf(fmaf(tForHi, tForHi, sHi * sHi * tf.y)));
    const float lo = 2.f * sLo * tf.w / (tForLo + sqrtf(fmaf(tForLo, tForLo, sLo * sLo * tf.y)));
    const float marg = 1e-4f * fmaxf(fabsf(lo), fabsf(hi)) +
                       1e-5f * (fabsf(m0) + fabsf(tf.x)) + 1e-3f;
    // NaN anywhere keeps the trace
    return !((m0 + lo) - marg > tf.x + apm || (m0 + hi) + marg < tf.x - apm);
}

// The same test for any h0.  With A = h^2 + h0^2, D = h^2 - h0^2 the
// reference's radicand satisfies tq^2 + tq ts gs + 16 h^2 h0^2 ts^2 =
// (tq + 2 theta^2 A)^2 - 4 theta^4 D^2 (gs = 4A, ts = theta^2), so
// sqrt(arg2) = sqrt(T^2 + 4 theta^2 H^2) + sqrt(T^2 + 4 theta^2 L^2) with
// T = t0^2 - c h0^2, H = max(|h|, |h0|), L = min(|h|, |h0|), and
//     mh - m0 = sign(D) G,  G = 2 theta |D| / sqrt(arg2).
// G increases with theta = t0 * slope and, for a fixed theta, moves toward 0
// as |T| grows, so over theta in [thLo, thHi] and |T| in [tLo, tHi] it lies
// between two corner values.  The box is taken over the lanes' own theta and
// T (the values their per-sample tests use); T must keep one sign and
// |T| >= kOctBoxMinT (the reference's tq^2 term stays normal), else the warp
// runs without the test.  H^2 and L^2 come from h and h0 directly (from the
// table, gs/2 - 2|D| would lose L^2 to cancellation when |h0| << |h|); D is
// the table's, as in the reference's numerator; margin as oct_box_may_pass.
constexpr float kOctBoxMinT = 1e-8f;
__device__ __forceinline__ float oct_box_g(float th, float T, float ad, float h4, float l4) {
    const float th2 = th * th;
    return 2.f * th * ad / (sqrtf(fmaf(T, T, th2 * h4)) + sqrtf(fmaf(T, T, th2 * l4)));
}
__device__ __forceinline__ bool oct_box_may_pass_h0(const float4 &tf, float h, float h0,
                                                    float thLo, float thHi, float tLo, float tHi,
                                                    float m0, float apm) {
    const float ad = fabsf(tf.w);
    const float hh = h * h, hh0 = h0 * h0;
    const float h4 = 4.f * fmaxf(hh, hh0), l4 = 4.f * fminf(hh, hh0);
    const float gHi = oct_box_g(thHi, thHi > 0.f ? tLo : tHi, ad, h4, l4);
    const float gLo = oct_box_g(thLo, thLo > 0.f ? tHi : tLo, ad, h4, l4);
    const float lo = tf.w >= 0.f ? gLo : -gHi, hi = tf.w >= 0.f ? gHi : -gLo;
    const float marg = 1e-4f * fmaxf(fabsf(lo), fabsf(hi)) +
                       1e-5f * (fabsf(m0) + fabsf(tf.x)) + 1e-3f;
    return !((m0 + lo) - marg > tf.x + apm || (m0 + hi) + marg < tf.x - apm);
}

// A warp's box for the displaced-midpoint test: h0 = 0 -- t0 and slope
// ranges of the members with t0 > 0 (t0 = 0 fails the per-sample test by
// itself: division by zero); otherwise theta and |T| ranges of the members.
// Called by all 32 lanes; member: the lane's evaluation counts.
struct OctWarpBox {
    bool on, h0zero;
    float aLo, aHi, bLo, bHi;  // h0 = 0: t0, slope; else theta, |T|
};
__device__ __forceinline__ OctWarpBox oct_warp_box(bool enable, bool member, float t0,
                                                   float slope, const OctCand &kc, float h0) {
    const float inf = __int_as_float(0x7f800000);
    OctWarpBox r;
    r.h0zero = h0 == 0.f;
    const bool in = member && (!r.h0zero || t0 > 0.f);
    const float a = r.h0zero ? t0 : 0.5f * kc.twoTheta;
    const float b = r.h0zero ? slope : kc.tn0_sq;
    // a NaN member (none with validated inputs) would pass every per-sample
    // test while fminf / fmaxf leave it out of the box: no box then
    const bool nan = in && (a != a || b != b);
    r.aLo = in ? a : inf;
    r.aHi = in ? a : -inf;
    r.bLo = in ? b : inf;
    r.bHi = in ? b : -inf;
    enable = enable && !__any_sync(0xffffffffu, nan);
#pragma unroll
    for (int sh = 16; sh; sh >>= 1) {
        r.aLo = fminf(r.aLo, __shfl_xor_sync(0xffffffffu, r.aLo, sh));
        r.aHi = fmaxf(r.aHi, __shfl_xor_sync(0xffffffffu, r.aHi, sh));
        r.bLo = fminf(r.bLo, __shfl_xor_sync(0xffffffffu, r.bLo, sh));
        r.bHi = fmaxf(r.bHi, __shfl_xor_sync(0xffffffffu, r.bHi, sh));
    }
    if (r.h0zero) {
        r.on = enable && r.aLo >= kOctBoxMinT0 && r.aHi >= r.aLo;
    } else {
        if (r.bHi < 0.f) {  // T < 0 throughout: |T| in [-bHi, -bLo]
            const float t = -r.bLo;
            r.bLo = -r.bHi;
            r.bHi = t;
        }
        r.on = enable && r.aHi >= r.aLo && r.bLo >= kOctBoxMinT && r.bHi >= r.bLo;
    }
    return r;
}
// Box test of trace ti for one t0 and a set of candidates whose slopes lie in
// [sLo, sHi] and whose c = 4/v^2 lie in [cLo, cHi] (trace selection: may any
// of them reach the trace at this t0?).  The candidates' theta = t0 * slope
// and T = t0^2 - c h0^2, rounded as their per-candidate tests round them, are
// monotone in slope and c, so the box is taken from the extremes; false only
// where the box test proves that no candidate passes.
__device__ __forceinline__ bool oct_sample_may_pass(const float4 &tf, float h, float h0,
                                                    float t0, float sLo, float sHi, float cLo,
                                                    float cHi, float m0, float apm) {
    if (h0 == 0.f) {
        if (!(t0 >= kOctBoxMinT0)) return true;  // the per-candidate tests decide
        return oct_box_may_pass(tf, sLo, sHi, t0, t0, m0, apm);
    }
    const float thLo = __fmul_rn(t0, sLo), thHi = __fmul_rn(t0, sHi);
    float tLo = oct_tn0_sq(t0, cHi, h0), tHi = oct_tn0_sq(t0, cLo, h0);
    if (tHi < 0.f) {  // T < 0 throughout: |T| in [-tHi, -tLo]
        const float t = -tLo;
        tLo = -tHi;
        tHi = t;
    }
    if (!(tLo >= kOctBoxMinT) || !(tHi >= tLo) || !(thHi >= thLo)) return true;
    return oct_box_may_pass_h0(tf, h, h0, thLo, thHi, tLo, tHi, m0, apm);
}

// Box test of trace ti (factor table entry and half-offset) for a warp.  The
// box {aLo, aHi, bLo, bHi} is read from the warp's slot in shared memory
// (volatile: reloaded at each test instead of held in registers through the
// trace loop).
// The OCT half-offset and factor table of midpoint mi of a launch (one h0,
// or the h0 block mi falls in).
struct OctLine {
    const float4 *tab;  // {m, gamma^2, 16h^2h0^2, h^2-h0^2} per trace
    float h0;
};
__device__ __forceinline__ OctLine oct_line(const LsParams &a, uint32_t mi) {
    OctLine l;
    if (a.m0PerH0 == 0) {
        l.tab = a.octTab;
        l.h0 = a.h0;
    } else {
        const uint32_t b = mi / a.m0PerH0;
        l.tab = a.octTab + (size_t)b * a.octTabStride;
        l.h0 = a.h0s[b];
    }
    return l;
}

// Window amplitudes y[0..n) of trace ti from sample k as FP32: the FP32 row,
// or the 16-bit row widened (BF16: the high half of an FP32 word; FP16:
// times the trace's scale).
__device__ __forceinline__ float amp16(const LsParams &a, uint32_t ti, uint16_t bits) {
    return a.storage == 2 ? __half2float(__ushort_as_half(bits)) * __ldg(a.scale + ti)
                          : __uint_as_float((uint32_t)bits << 16);
}
template <int N>
__device__ __forceinline__ void load_window(const LsParams &a, uint32_t ti, int k, float (&y)[N]) {
    if (a.samples16) {
        const uint16_t *r = a.samples16 + (size_t)ti * a.stride + k;
        const float sc = a.storage == 2 ? __ldg(a.scale + ti) : 1.f;
#pragma unroll
        for (int j = 0; j < N; j++) {
            const uint16_t b = __ldg(r + j);
            y[j] = a.storage == 2 ? __half2float(__ushort_as_half(b)) * sc
                                  : __uint_as_float((uint32_t)b << 16);
        }
    } else {
        const float *r = a.samples + (size_t)ti * a.stride + k;
#pragma unroll
        for (int j = 0; j < N; j++) y[j] = __ldg(r + j);
    }
}
// The W taps of the window of trace ti starting at sample k with fraction
// frac, added to the sums (COMPUTE_SEMBLANCE, interface.h:26-44): each
// amplitude loaded as its tap needs it (one live value, not W + 1).
template <int W>
__device__ __forceinline__ void accum_window(const LsParams &a, uint32_t ti, int k, float frac,
                                             float (&num)[W], float &lin, float &den) {
    if (a.samples16) {
        const uint16_t *r = a.samples16 + (size_t)ti * a.stride + k;
        const float sc = a.storage == 2 ? __ldg(a.scale + ti) : 1.f;
        auto wid = [&](uint16_t b) {
            return a.storage == 2 ? __half2float(__ushort_as_half(b)) * sc
                                  : __uint_as_float((uint32_t)b << 16);
        };
        float y1 = wid(__ldg(r));
#pragma unroll
        for (int j = 0; j < W; j++) {
            const float y0 = y1;
            y1 = wid(__ldg(r + j + 1));
            const float u = (y1 - y0) * frac + y0;
            num[j] += u;
            lin += u;
            den += u * u;
        }
    } else {
        const float *r = a.samples + (size_t)ti * a.stride + k;
        float y1 = __ldg(r);
#pragma unroll
        for (int j = 0; j < W; j++) {
            const float y0 = y1;
            y1 = __ldg(r + j + 1);
            const float u = (y1 - y0) * frac + y0;
            num[j] += u;
            lin += u;
            den += u * u;
        }
    }
}

// One amplitude (runtime-sized windows).
__device__ __forceinline__ float amp_at(const LsParams &a, uint32_t ti, int k) {
    return a.samples16 ? amp16(a, ti, __ldg(a.samples16 + (size_t)ti * a.stride + k))
                       : __ldg(a.samples + (size_t)ti * a.stride + k);
}

__device__ __forceinline__ void oct_box_store(volatile float *slot, const OctWarpBox &r) {
    slot[0] = r.aLo;
    slot[1] = r.aHi;
    slot[2] = r.bLo;
    slot[3] = r.bHi;
    __syncwarp();
}
// The warp box test of one trace, with its table entry and half-offset given.
__device__ __forceinline__ bool oct_box_keep_tf(const LsParams &a, const OctLine &ol, float4 tf,
                                                float hoff, const volatile float *slot,
                                                float m0) {
    const float aLo = slot[0], aHi = slot[1], bLo = slot[2], bHi = slot[3];
    return ol.h0 == 0.f ? oct_box_may_pass(tf, bLo, bHi, aLo, aHi, m0, a.apm)
                        : oct_box_may_pass_h0(tf, hoff, ol.h0, aLo, aHi, bLo, bHi, m0, a.apm);
}
__device__ __forceinline__ bool oct_box_keep(const LsParams &a, const OctLine &ol, uint32_t ti,
                                             const volatile float *slot, float m0) {
    const float4 tf = __ldg(ol.tab + ti);
    const float aLo = slot[0], aHi = slot[1], bLo = slot[2], bHi = slot[3];
    return ol.h0 == 0.f ? oct_box_may_pass(tf, bLo, bHi, aLo, aHi, m0, a.apm)
                        : oct_box_may_pass_h0(tf, __ldg(a.hoff + ti), ol.h0, aLo, aHi, bLo, bHi,
                                              m0, a.apm);
}

// Where oct_eval_traces takes trace b's table entry, half-offset and index
// from: the line in global memory (trace indices tb) ...
template <int B>
struct OctGlobalTraces {
    const float4 *tab;
    const float *hoffs;
    uint32_t tb[B];
    __device__ __forceinline__ float4 entry(int b) const { return __ldg(tab + tb[b]); }
    __device__ __forceinline__ float hoff(int b) const { return hoffs[tb[b]]; }
    __device__ __forceinline__ uint32_t index(int b) const { return tb[b]; }
};
// ... or a warp's block of 32 traces copied to shared memory by its box test
// (slots bit[b] of the block)
template <int B>
struct OctBlockTraces {
    const float4 *tab;
    const float *hoffs;
    const uint32_t *ti;
    uint32_t bit[B];
    __device__ __forceinline__ float4 entry(int b) const { return tab[bit[b]]; }
    __device__ __forceinline__ float hoff(int b) const { return hoffs[bit[b]]; }
    __device__ __forceinline__ uint32_t index(int b) const { return ti[bit[b]]; }
};

// B traces of one thread's OCT candidate (factors kc, c = 4/v^2, slope):
// the displaced-midpoint tests side by side (independent chains), then time
// and window of the passing traces in order, as COMPUTE_SEMBLANCE
// (interface.h:26-44).  live[b] false: padding, neither evaluated nor
// counted.
template <int W, int B, typename Traces>
__device__ __forceinline__ void oct_eval_traces(const LsParams &a, const OctLine &ol,
                                                const Traces &tr, const bool (&live)[B],
                                                const OctCand &kc, float c, float slope,
                                                float t0, float m0, float (&num)[W], float &lin,
                                                float &den, unsigned &used, unsigned &nu) {
    float4 fb[B];  // {m, gamma^2, 16h^2h0^2, h^2-h0^2}
    float mhb[B];
    bool pass[B];
#pragma unroll
    for (int b = 0; b < B; b++) fb[b] = tr.entry(b);
#pragma unroll
    for (int b = 0; b < B; b++) {
        const int e = oct_mh_all(kc, fb[b].y, fb[b].z, fb[b].w, m0, &mhb[b]);
        pass[b] = e == DE_OK && !(fabsf(fb[b].x - mhb[b]) > a.apm);
    }
#pragma unroll
    for (int b = 0; b < B; b++) {
        if (!live[b]) continue;
        if (!pass[b]) {
            nu++;
            continue;
        }
        float t;
        if (oct_time_k(tr.hoff(b), ol.h0, t0, kc.tn0_sq, m0, fb[b].x, mhb[b], c, slope, &t) !=
            DE_OK)
            continue;
        const WinIdx wi = window_index(t, a.dt);
        if (window_in_trace(wi.k, a.tau, (int)a.S)) {
            accum_window<W>(a, tr.index(b), wi.k - a.tau, wi.frac, num, lin, den);
            used++;
        }
    }
}

// oct_eval_traces over traces tb of the line in global memory.
template <int W, int B>
__device__ __forceinline__ void oct_eval_batch(const LsParams &a, const OctLine &ol,
                                               const uint32_t (&tb)[B],
                                               const bool (&live)[B], const OctCand &kc,
                                               float c, float slope, float t0, float m0,
                                               float (&num)[W], float &lin, float &den,
                                               unsigned &used, unsigned &nu) {
    OctGlobalTraces<B> tr;
    tr.tab = ol.tab;
    tr.hoffs = a.hoff;
#pragma unroll
    for (int b = 0; b < B; b++) tr.tb[b] = tb[b];
    oct_eval_traces<W, B>(a, ol, tr, live, kc, c, slope, t0, m0, num, lin, den, used, nu);
}

}  // namespace hpss
