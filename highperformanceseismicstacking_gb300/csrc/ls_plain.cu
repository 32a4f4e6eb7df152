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

template <int MODEL>
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
        for (uint32_t q = 0; q < cnt; q++) {
            const uint32_t ti = a.selIdx ? a.selIdx[first + q] : first + q;
            float t;
            int ok = model_time<MODEL>(t0, c, p1, p2, a.mid[ti], a.hoff[ti],
                                       a.hsq[ti], m0, a.apm, a.h0, &t);
            if (ok < 0) {
                nu++;
                continue;
            }
            if (ok == 0) continue;
            const float *tr = a.samples + (size_t)ti * a.stride;
            WinIdx wi = window_index(t, a.dt);
            if (window_in_trace(wi.k, a.tau, (int)a.S)) {
                int k = wi.k - a.tau;
                float y1 = tr[k];
                for (int j = 0; j < a.w; j++, k++) {
                    float y0 = y1;
                    y1 = tr[k + 1];
                    float u = (y1 - y0) * wi.frac + y0;
                    num[j] += u;
                    lin += u;
                    den += u * u;
                }
                used++;
            }
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

cudaError_t launch_ls_plain(const LsParams &p, cudaStream_t st) {
    if (p.nM0 == 0 || p.S == 0) return cudaSuccess;
    const uint64_t blocks = (uint64_t)p.nM0 * p.S;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    switch (p.np == 1 ? kModelCmp : (p.np == 3 ? kModelZocrs : kModelOct)) {
        case kModelCmp:
            ls_plain_kernel<kModelCmp><<<(unsigned)blocks, kPlainThreads, 0, st>>>(p);
            break;
        case kModelZocrs:
            ls_plain_kernel<kModelZocrs><<<(unsigned)blocks, kPlainThreads, 0, st>>>(p);
            break;
        default:
            ls_plain_kernel<kModelOct><<<(unsigned)blocks, kPlainThreads, 0, st>>>(p);
            break;
    }
    return cudaGetLastError();
}

}  // namespace hpss
