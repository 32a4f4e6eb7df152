// ls_plain.cu -- the plain FP32 linear-search kernel.
//
// One thread per (t0 sample, candidate), traces read from global memory, a
// runtime-sized window accumulator -- the form of the reference kernels
// computeSemblancesFor{CommonMidPoint,ZeroOffsetCommonReflectionSurface,
// OffsetContinuationTrajectory} (cuda/src/semblance/kernel/{cmp,zocrs,oct}/
// linear_search.cu) with the same arithmetic, so its semblance, stack and
// selected candidate are bit-identical to the reference's.  Unlike the
// reference it keeps no [S][P] semblance/stack intermediates: a CTA owns one
// (midpoint, sample) pair, loops its threads over the candidates and reduces
// the argmax in shared memory (selectBestSemblancesFor*, same tie rule).
// All midpoints of a call run in one launch.
#include "hpss_device.cuh"
#include "hpss_internal.h"

namespace hpss {

// ---- precision modes (no reference counterpart; plain kernel only) -------
//
// kPrecTt64: the ZO-CRS / OCT traveltime is formed in FP64 from the FP32
//   inputs (square-root arguments, divisions, the displaced midpoint) and
//   rounded to FP32 once; the window arithmetic stays FP32.
// kPrecCompensated: when window x selected traces exceeds 4096 terms, the
//   window sums (numerator per tap, linear sum, denominator) are accumulated
//   with Neumaier's compensated summation (Neumaier 1974, the improved
//   Kahan-Babuska sum): sum + compensation, the compensation added once at
//   the end.

// Neumaier step: s + x with the rounding error of the add kept in comp.
__device__ __forceinline__ void neumaier(float &s, float &comp, float x) {
    const float t = __fadd_rn(s, x);
    comp = __fadd_rn(comp, fabsf(s) >= fabsf(x) ? __fadd_rn(__fsub_rn(s, t), x)
                                                : __fadd_rn(__fsub_rn(x, t), s));
    s = t;
}

constexpr int kCompensateAbove = 4096;  // window x traces terms

// S16: the line is stored in 16-bit rows (widened as read); a template
// parameter so that the FP32 form carries no per-tap storage test.
template <int MODEL, int MODE, bool S16>
__global__ void __launch_bounds__(kPlainThreads)
ls_plain_kernel(LsParams a) {
    const uint32_t mi = blockIdx.x / a.S;
    const uint32_t s = blockIdx.x % a.S;
    if (mi >= a.nM0) return;
    const float m0 = a.m0s[mi];
    const uint32_t first = a.selFirst[mi], cnt = a.selCount[mi];
    const int np = a.np;
    float *out = a.out + (size_t)mi * (2 + np) * a.S;

    // No selected trace: the reference skips the midpoint and returns its
    // reset (all-zero) result array (CudaLinearSearchAlgorithm.cu:37-40).
    if (cnt == 0) {
        if (threadIdx.x < 2 + np) out[(size_t)threadIdx.x * a.S + s] = 0.f;
        return;
    }

    const float t0 = static_cast<float>(s) * a.dt;
    const float h0 = MODEL == kModelOct ? oct_line(a, mi).h0 : 0.f;
    float best = -1.f, bestStack = 0.f, second = -1.f;
    uint32_t bestP = 0xffffffffu;
    unsigned long long notUsed = 0;

    for (uint32_t p = threadIdx.x; p < a.P; p += blockDim.x) {
        const float *pr = a.params + (size_t)p * np;
        const float c = pr[0];
        const float p1 = np > 1 ? pr[1] : 0.f;
        const float p2 = np > 2 ? pr[2] : 0.f;
        float num[kMaxWindow + 1];
        float lin = 0.f, den = 0.f;
        unsigned used = 0, nu = 0;
        for (int j = 0; j < a.w; j++) num[j] = 0.f;
        // compensated sums (MODE & kPrecCompensated, large windows x traces)
        constexpr bool kMayComp = (MODE & kPrecCompensated) != 0;
        const bool comp = kMayComp && (uint64_t)a.w * cnt > (uint64_t)kCompensateAbove;
        float numc[kMayComp ? kMaxWindow + 1 : 1];
        float linc = 0.f, denc = 0.f;
        if (kMayComp)
            for (int j = 0; j < a.w; j++) numc[j] = 0.f;
        for (uint32_t q = 0; q < cnt; q++) {
            const uint32_t ti = a.selIdx ? a.selIdx[first + q] : first + q;
            float t;
            int ok;
            if ((MODE & kPrecTt64) && MODEL == kModelZocrs)
                ok = zocrs_time_tt64(t0, c, p1, p2, a.mid[ti] - m0, a.hsq[ti], &t) ? 1 : 0;
            else if ((MODE & kPrecTt64) && MODEL == kModelOct)
                ok = oct_time_f64(t0, c, p1, a.mid[ti], a.hoff[ti], m0, a.apm, h0, &t);
            else
                ok = model_time<MODEL>(t0, c, p1, p2, a.mid[ti], a.hoff[ti], a.hsq[ti], m0,
                                       a.apm, h0, &t);
            if (ok < 0) {
                nu++;
                continue;
            }
            if (ok == 0) continue;
            WinIdx wi = window_index(t, a.dt);
            if (window_in_trace(wi.k, a.tau, (int)a.S)) {
                int k = wi.k - a.tau;
                const float *tr = a.samples + (size_t)ti * a.stride;
                const uint16_t *tr16 = a.samples16 + (size_t)ti * a.stride;
                float y1 = S16 ? amp16(a, ti, tr16[k]) : tr[k];
                for (int j = 0; j < a.w; j++, k++) {
                    float y0 = y1;
                    y1 = S16 ? amp16(a, ti, tr16[k + 1]) : tr[k + 1];
                    float u = (y1 - y0) * wi.frac + y0;
                    if (kMayComp && comp) {
                        neumaier(num[j], numc[j], u);
                        neumaier(lin, linc, u);
                        neumaier(den, denc, __fmul_rn(u, u));
                    } else {
                        num[j] += u;
                        lin += u;
                        den += u * u;
                    }
                }
                used++;
            }
        }
        if (kMayComp && comp) {
            for (int j = 0; j < a.w; j++) num[j] = __fadd_rn(num[j], numc[j]);
            lin = __fadd_rn(lin, linc);
            den = __fadd_rn(den, denc);
        }
        float sembl, stack;
        reduce_semblance(num, lin, den, a.w, used, &sembl, &stack);
        top2_offer(sembl, best, second);
        if (sembl > best) {
            best = sembl;
            bestStack = stack;
            bestP = p;
        }
        notUsed += nu;
    }

    // CTA argmax (lowest candidate index wins ties).
    __shared__ float shS[kPlainThreads / 32], shK[kPlainThreads / 32], sh2[kPlainThreads / 32];
    __shared__ uint32_t shP[kPlainThreads / 32];
    __shared__ unsigned long long shNu[kPlainThreads / 32];
    for (int o = 16; o; o >>= 1) {
        float os = __shfl_down_sync(0xffffffffu, best, o);
        float ok = __shfl_down_sync(0xffffffffu, bestStack, o);
        uint32_t op = __shfl_down_sync(0xffffffffu, bestP, o);
        float o2 = __shfl_down_sync(0xffffffffu, second, o);
        unsigned long long on = __shfl_down_sync(0xffffffffu, notUsed, o);
        const bool take = better(os, op, best, bestP);
        top2_merge(os, op, o2, best, bestP, second);
        if (take) bestStack = ok;
        notUsed += on;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        shS[warp] = best;
        shK[warp] = bestStack;
        shP[warp] = bestP;
        sh2[warp] = second;
        shNu[warp] = notUsed;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int wv = 1; wv < kPlainThreads / 32; wv++) {
            if (better(shS[wv], shP[wv], best, bestP)) bestStack = shK[wv];
            top2_merge(shS[wv], shP[wv], sh2[wv], best, bestP, second);
            notUsed += shNu[wv];
        }
        if (a.nearTies && near_tie(best, second)) atomicAdd(a.nearTies, 1ull);
        out[s] = best;
        out[a.S + s] = bestStack;
        if (bestP != 0xffffffffu) {
            const float *pr = a.params + (size_t)bestP * np;
            out[2 * a.S + s] = 2 / sqrtf(pr[0]);
            for (int j = 1; j < np; j++) out[(size_t)(2 + j) * a.S + s] = pr[j];
        } else {
            for (int j = 0; j < np; j++) out[(size_t)(2 + j) * a.S + s] = 0.f;
        }
        if (MODEL == kModelOct && a.notUsed && notUsed)
            atomicAdd(a.notUsed + mi, notUsed);
    }
}

template <int MODEL, bool S16>
void launch_plain_mode_s(const LsParams &p, unsigned blocks, int mode, cudaStream_t st) {
    switch (mode & (kPrecTt64 | kPrecCompensated)) {
        case 0: ls_plain_kernel<MODEL, 0, S16><<<blocks, kPlainThreads, 0, st>>>(p); break;
        case kPrecTt64:
            ls_plain_kernel<MODEL, kPrecTt64, S16><<<blocks, kPlainThreads, 0, st>>>(p);
            break;
        case kPrecCompensated:
            ls_plain_kernel<MODEL, kPrecCompensated, S16><<<blocks, kPlainThreads, 0, st>>>(p);
            break;
        default:
            ls_plain_kernel<MODEL, kPrecTt64 | kPrecCompensated, S16>
                <<<blocks, kPlainThreads, 0, st>>>(p);
            break;
    }
}

template <int MODEL>
void launch_plain_mode(const LsParams &p, unsigned blocks, int mode, cudaStream_t st) {
    if (p.samples16) launch_plain_mode_s<MODEL, true>(p, blocks, mode, st);
    else launch_plain_mode_s<MODEL, false>(p, blocks, mode, st);
}

cudaError_t launch_ls_plain(const LsParams &p, cudaStream_t st, int precisionMode) {
    if (p.nM0 == 0 || p.S == 0) return cudaSuccess;
    const uint64_t blocks = (uint64_t)p.nM0 * p.S;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    switch (p.np == 1 ? kModelCmp : (p.np == 3 ? kModelZocrs : kModelOct)) {
        case kModelCmp:
            launch_plain_mode<kModelCmp>(p, (unsigned)blocks, precisionMode, st);
            break;
        case kModelZocrs:
            launch_plain_mode<kModelZocrs>(p, (unsigned)blocks, precisionMode, st);
            break;
        default:
            launch_plain_mode<kModelOct>(p, (unsigned)blocks, precisionMode, st);
            break;
    }
    return cudaGetLastError();
}

}  // namespace hpss
