// sf.cu -- stretch-free stack (StretchFreeAlgorithm, common/src/semblance/
// algorithm/StretchFreeAlgorithm.cpp:23-125; kernels cuda/src/semblance/
// kernel/{cmp,zocrs,oct}/stretch_free.cu and common/stretch_free.cu).
//
// For every (midpoint, t0 sample s) and n in [-nmax, nmax] the parameters a
// previous search chose at sample s - n are applied at t0 = (s - n) dt and the
// traveltime is shifted by n dt; the window semblance and stack follow, and
// the n with the highest semblance is kept (strict '>' over n ascending, so
// the most negative n wins ties).  A warp owns one sample, its lanes the n
// values.  The reference runs only CMP on CUDA (its OCT case falls through
// into `throw`, CudaStretchFreeAlgorithm.cu:86-110); all three models run
// here, with the same per-model traveltime arithmetic as the searches.
#include "hpss_device.cuh"
#include "hpss_internal.h"

namespace hpss {

constexpr int kSfWarps = 8;

template <int MODEL>
__global__ void __launch_bounds__(kSfWarps * 32) sf_kernel(LsParams a, uint32_t nUnits) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int NP = MODEL == kModelCmp ? 1 : (MODEL == kModelZocrs ? 3 : 2);
    const int nn = 2 * a.nmax + 1;
    for (uint32_t unit = blockIdx.x * kSfWarps + warp; unit < nUnits;
         unit += gridDim.x * kSfWarps) {
        const uint32_t mi = unit / a.S;
        const int s = (int)(unit % a.S);
        const float m0 = a.m0s[mi];
        const uint32_t first = a.selFirst[mi], cnt = a.selCount[mi];
        const float *prior = a.prior + (size_t)mi * NP * a.S;
        float best = -1.f, bestK = 0.f;
        uint32_t bestI = 0xffffffffu;
        unsigned nu = 0;
        for (int ni0 = 0; ni0 < nn; ni0 += 32) {
            const int ni = ni0 + lane;
            const int n = ni - a.nmax;
            const int sn = s - n;
            float sembl = 0.f, stack = 0.f;
            if (ni < nn && sn >= 0 && sn < (int)a.S) {
                const float t0n = static_cast<float>(sn) * a.dt;
                const float v = prior[sn];
                const float c = 4.0f / (v * v);
                const float p1 = MODEL != kModelCmp ? prior[a.S + sn] : 0.f;
                const float p2 = MODEL == kModelZocrs ? prior[2 * a.S + sn] : 0.f;
                const float nf = static_cast<float>(n);
                float num[kMaxWindow + 1];
                for (int j = 0; j < a.w; j++) num[j] = 0.f;
                float lin = 0.f, den = 0.f;
                unsigned used = 0;
                for (uint32_t q = 0; q < cnt; q++) {
                    const uint32_t ti = a.selIdx ? a.selIdx[first + q] : first + q;
                    float tn;
                    int ok = model_time<MODEL>(t0n, c, p1, p2, a.mid[ti], a.hoff[ti], a.hsq[ti],
                                               m0, a.apm, a.h0, &tn);
                    if (ok < 0) {
                        nu++;
                        continue;
                    }
                    if (ok == 0) continue;
                    // t_n + n dt as one fused multiply-add, as the reference
                    // compiles it (cmp/stretch_free.cu:55)
                    const float t = __fmaf_rn(nf, a.dt, tn);
                    WinIdx wi = window_index(t, a.dt);
                    if (window_in_trace(wi.k, a.tau, (int)a.S)) {
                        const float *tr = a.samples + (size_t)ti * a.stride + (wi.k - a.tau);
                        float y1 = __ldg(tr);
                        for (int j = 0; j < a.w; j++) {
                            float y0 = y1;
                            y1 = __ldg(tr + j + 1);
                            float u = (y1 - y0) * wi.frac + y0;
                            num[j] += u;
                            lin += u;
                            den += u * u;
                        }
                        used++;
                    }
                }
                reduce_semblance(num, lin, den, a.w, used, &sembl, &stack);
            }
            if (ni < nn && sembl > best) {
                best = sembl;
                bestK = stack;
                bestI = (uint32_t)ni;
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            float os = __shfl_xor_sync(0xffffffffu, best, o);
            float ok = __shfl_xor_sync(0xffffffffu, bestK, o);
            uint32_t oi = __shfl_xor_sync(0xffffffffu, bestI, o);
            if (better(os, oi, best, bestI)) {
                best = os;
                bestK = ok;
                bestI = oi;
            }
            nu += __shfl_xor_sync(0xffffffffu, nu, o);
        }
        if (lane == 0) {
            float *out = a.out + (size_t)mi * 3 * a.S;
            out[s] = best;
            out[a.S + s] = bestK;
            out[2 * a.S + s] = bestI != 0xffffffffu ? (float)((int)bestI - a.nmax) : 0.f;
            if (MODEL == kModelOct && a.notUsed && nu)
                atomicAdd(a.notUsed + mi, (unsigned long long)nu);
        }
    }
}

// OCT trace selection with the prior parameters of every sample
// (selectTracesForOffsetContinuationTrajectory, oct/stretch_free.cu:99-138).
__global__ void sf_select_oct_kernel(LsParams a, const uint32_t *candFirst,
                                     const uint32_t *candCount, uint32_t *selIdx,
                                     uint32_t *selCount) {
    const uint32_t mi = blockIdx.x;
    const float m0 = a.m0s[mi];
    const float *prior = a.prior + (size_t)mi * 2 * a.S;
    const uint32_t first = candFirst[mi], count = candCount[mi];
    const uint32_t outBase = a.selFirst[mi];
    __shared__ uint32_t shCount;
    __shared__ uint32_t shFlags[256];
    if (threadIdx.x == 0) shCount = 0;
    __syncthreads();
    for (uint32_t base = 0; base < count; base += blockDim.x) {
        const uint32_t q = base + threadIdx.x;
        bool used = false;
        if (q < count) {
            const uint32_t ti = first + q;
            const float m = a.mid[ti], h = a.hoff[ti];
            for (uint32_t s = 0; s < a.S && !used; s++) {
                const float t0 = static_cast<float>(s) * a.dt;
                const float v = prior[s];
                const float c = 4.0f / (v * v);
                float mh;
                int e = oct_displaced_midpoint(h, a.h0, t0, m0, c, prior[a.S + s], &mh);
                used = (e == DE_OK && fabsf(m - mh) <= a.apm);
            }
        }
        shFlags[threadIdx.x] = used ? 1u : 0u;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (uint32_t w = 0; w < blockDim.x && base + w < count; w++)
                if (shFlags[w]) selIdx[outBase + shCount++] = first + base + w;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) selCount[mi] = shCount;
}

cudaError_t launch_sf(const LsParams &p, int model, uint32_t grid, uint32_t nUnits,
                      cudaStream_t st) {
    if (model == kModelCmp)
        sf_kernel<kModelCmp><<<grid, kSfWarps * 32, 0, st>>>(p, nUnits);
    else if (model == kModelZocrs)
        sf_kernel<kModelZocrs><<<grid, kSfWarps * 32, 0, st>>>(p, nUnits);
    else
        sf_kernel<kModelOct><<<grid, kSfWarps * 32, 0, st>>>(p, nUnits);
    return cudaGetLastError();
}

cudaError_t launch_sf_select_oct(const LsParams &p, const uint32_t *candFirst,
                                 const uint32_t *candCount, uint32_t *selIdx,
                                 uint32_t *selCount, cudaStream_t st) {
    if (p.nM0 == 0) return cudaSuccess;
    sf_select_oct_kernel<<<p.nM0, 256, 0, st>>>(p, candFirst, candCount, selIdx, selCount);
    return cudaGetLastError();
}

}  // namespace hpss
