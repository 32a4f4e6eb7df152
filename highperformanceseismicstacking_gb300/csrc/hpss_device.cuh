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

#include <cstdint>

#include "hpss_internal.h"

namespace hpss {

// gpu_error_code (common/include/gpu/interface.h:12-18).
enum DevErr : int { DE_OK = 0, DE_DIV_ZERO = 1, DE_NEG_SQRT = 2 };

// CMP: t = sqrt(t0^2 + c h^2), c = 4/v^2 (cmp/linear_search.cu:57).
__device__ __forceinline__ float cmp_time(float t0, float c, float h_sq) {
    return sqrtf(t0 * t0 + c * h_sq);
}

// ZO-CRS: t^2 = (t0 + A dm)^2 + B dm^2 + C h^2 (zocrs/linear_search.cu:83-87).
// Returns false when the squared time is negative (window skipped).
__device__ __forceinline__ bool zocrs_time(float t0, float c, float a, float b,
                                           float dm, float h_sq, float *t) {
    float tmp = t0 + a * dm;
    tmp = tmp * tmp + b * dm * dm + c * h_sq;
    if (tmp >= 0) {
        *t = sqrtf(tmp);
        return true;
    }
    return false;
}

// OCT displaced midpoint (oct/common.cuh:7-35).
__device__ __forceinline__ int oct_displaced_midpoint(float h, float h0,
                                                      float t0, float m0,
                                                      float c, float slope,
                                                      float *mh) {
    float theta = t0 * slope;
    float gamma = 2 * sqrtf(h * h + h0 * h0);
    float tn0_sq = t0 * t0 - c * h0 * h0;
    float theta_sq = theta * theta;
    float gamma_sq = gamma * gamma;
    float tn0_quad = tn0_sq * tn0_sq;
    float arg = tn0_quad * tn0_quad + tn0_quad * theta_sq * gamma_sq +
                16 * h * h * h0 * h0 * theta_sq * theta_sq;
    if (arg < 0) return DE_NEG_SQRT;
    arg = theta_sq * gamma_sq + 2 * tn0_quad + 2 * sqrtf(arg);
    if (arg == 0) return DE_DIV_ZERO;
    *mh = m0 + 2 * theta * (h * h - h0 * h0) / sqrtf(arg);
    return DE_OK;
}

// OCT traveltime at the displaced midpoint (oct/common.cuh:37-94).
__device__ __forceinline__ int oct_time(float h, float h0, float t0, float m0,
                                        float m, float mh, float c,
                                        float slope, float *out) {
    float tn0_sq = t0 * t0 - c * h0 * h0;
    float w1 = (h + h0) * (h + h0) - (mh - m0) * (mh - m0);
    float w2 = (h - h0) * (h - h0) - (mh - m0) * (mh - m0);
    if (w1 < 0 || w2 < 0) return DE_NEG_SQRT;
    float u = sqrtf(w1) + sqrtf(w2);
    float th = t0;
    if (fabsf(h) > fabsf(h0)) {
        if (!u) return DE_DIV_ZERO;
        float arg = c * h * h + 4 * h * h / (u * u) * tn0_sq;
        if (arg < 0) return DE_NEG_SQRT;
        th = sqrtf(arg);
    } else if (fabsf(h) < fabsf(h0)) {
        if (!h0) return DE_DIV_ZERO;
        float arg = c * h * h + u * u / (4 * h0 * h0) * tn0_sq;
        if (arg < 0) return DE_NEG_SQRT;
        th = sqrtf(arg);
    }
    float tn_sq = th * th - c * h * h;
    if (!th || !tn0_sq) return DE_DIV_ZERO;
    float ah = (t0 * tn_sq) / (th * tn0_sq) * slope;
    *out = th + ah * (m - mh);
    return DE_OK;
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
        float mh;
        int e = oct_displaced_midpoint(h, h0, t0, m0, c, p1, &mh);
        if (e != DE_OK || fabsf(m - mh) > apm) return -1;
        e = oct_time(h, h0, t0, m0, m, mh, c, p1, t);
        return e == DE_OK ? 1 : 0;
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

}  // namespace hpss
