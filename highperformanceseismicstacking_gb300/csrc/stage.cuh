// stage.cuh -- staging of trace sample spans into shared memory, shared by
// the tuned linear-search kernel (ls_tuned.cuh) and the differential
// evolution (de.cu): the span of a trace that any window of a parameter box
// and a t0 range can touch, and bulk (TMA) copies completing on an mbarrier
// with a bounded wait.
#pragma once

#include <cuda_fp16.h>

#include "hpss_device.cuh"
#include "hpss_internal.h"

namespace hpss {

// Sample span [lo, lo+len) of trace (m, h, hsq) touched by any in-trace
// window of the tile [t0a, t0b] and the chunk parameter box.  Conservative by
// one sample each side; rounded to multiples of ALIGN samples (4: 16 bytes
// of FP32; 8: 16 bytes of 16-bit rows, whose stride is a multiple of 8) for
// bulk copies.  len = 0 if no window of the tile/chunk can lie inside the trace.
// *full (optional): every window of the tile and chunk box lies inside the
// trace (for ZO-CRS also: every squared time is positive), judged on the same
// conservative bounds, so the evaluation may skip the per-candidate checks.
template <int MODEL, int ALIGN = 4>
__device__ __forceinline__ void trace_span(const LsParams &a, const float *cb,
                                           float m0, float t0a, float t0b,
                                           float m, float hsq, int *lo,
                                           int *len, bool *full = nullptr) {
    const int S = (int)a.S, tau = a.tau;
    int kmin, kmax;
    bool positive = true;
    if (MODEL == kModelCmp) {
        // t increases with t0 and with c
        kmin = window_index(cmp_time(t0a, cb[0], hsq), a.dt).k - 1;
        kmax = window_index(cmp_time(t0b, cb[1], hsq), a.dt).k + 1;
    } else if (MODEL == kModelZocrs) {
        const float dm = m - m0;
        float x1 = cb[2] * dm, x2 = cb[3] * dm;
        float xlo = t0a + fminf(x1, x2), xhi = t0b + fmaxf(x1, x2);
        float x2min = (xlo <= 0.f && xhi >= 0.f) ? 0.f : fminf(xlo * xlo, xhi * xhi);
        float x2max = fmaxf(xlo * xlo, xhi * xhi);
        float dm2 = dm * dm;
        float b1 = cb[4] * dm2, b2 = cb[5] * dm2;
        float c1 = cb[0] * hsq, c2 = cb[1] * hsq;
        float tlo = x2min + fminf(b1, b2) + fminf(c1, c2);
        float thi = x2max + fmaxf(b1, b2) + fmaxf(c1, c2);
        if (thi < 0.f) {
            *lo = 0;
            *len = 0;
            if (full) *full = false;
            return;
        }
        positive = tlo > 1e-4f * thi;
        // relative slack for the different summation order of the kernel
        tlo = fmaxf(tlo, 0.f) * 0.9999f;
        thi = thi * 1.0001f;
        kmin = window_index(sqrtf(tlo), a.dt).k - 2;
        kmax = window_index(sqrtf(thi), a.dt).k + 2;
    } else {
        kmin = tau;
        kmax = S - tau - 2;
        positive = false;
    }
    if (full) *full = positive && kmin >= tau && kmax <= S - tau - 2;
    // in-trace windows have tau <= k <= S - tau - 2
    kmin = max(kmin, tau);
    kmax = min(kmax, S - tau - 2);
    if (kmin > kmax) {
        *lo = 0;
        *len = 0;
        if (full) *full = false;
        return;
    }
    int l = (kmin - tau) & ~(ALIGN - 1);
    int h = kmax + tau + 1;                                      // last sample read
    int e = min((h + ALIGN) & ~(ALIGN - 1), (int)a.stride);      // exclusive, multiple of ALIGN
    *lo = l;
    *len = e - l;
}

// Bulk (TMA) copies of FP32 trace spans into a stage.  One thread
// registers the round's byte count on the mbarrier; the lane that owns a
// span issues one cp.async.bulk for it (16-byte aligned addresses, size a
// multiple of 16 bytes), which counts its bytes off the same barrier.
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void stage_bar_init(unsigned long long *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void stage_bar_expect(unsigned long long *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void stage_bulk_copy(void *dst, const void *src, uint32_t bytes,
                                                unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// true once the barrier's phase `parity` has completed
__device__ __forceinline__ bool stage_bar_try_wait(unsigned long long *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Bounded wait for phase `parity`; false when it did not complete within
// `limit` polls.
__device__ __forceinline__ bool stage_bar_wait(unsigned long long *bar, uint32_t parity,
                                               uint32_t limit) {
    for (uint32_t it = 0; it < limit; it++)
        if (stage_bar_try_wait(bar, parity)) return true;
    return false;
}

// 16-bit FP16 bits widened to FP32
__device__ __forceinline__ float half_bits_to_float(unsigned bits) {
    return __half2float(__ushort_as_half((unsigned short)bits));
}

}  // namespace hpss
