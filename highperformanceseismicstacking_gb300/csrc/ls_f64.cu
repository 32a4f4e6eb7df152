// ls_f64.cu -- the linear search with every step in FP64 (precision mode
// HPSS_PREC_FP64; no reference counterpart).
//
// The traveltime, the window index and fraction, the interpolation, the
// window sums, the semblance and the argmax are all FP64, in the operation
// order of the FP64 instantiation of the host oracle (the reference's
// COMPUTE_SEMBLANCE / REDUCE_SEMBLANCE_STACK, interface.h:26-55, and the OCT
// helpers, oct/common.cuh:7-94, evaluated in double), so that a
// workload-size sample -- 10^4 (m0, t0) samples of the 21 x 21 x 41 ZO-CRS
// grid, some 3.5e11 evaluations, far beyond what the host oracle can run --
// has an FP64 reference for the FP32 modes.  One CTA per (midpoint, t0
// sample), threads over the candidates, as the plain kernel; the results are
// rounded to FP32 once, and the near-tie count uses the FP64 semblances.
#include "hpss_device.cuh"
#include "hpss_internal.h"

namespace hpss {

// One trace of one (t0, candidate) in FP64: traveltime (+ the stretch-free
// shift), window and sums, as the FP64 oracle's eval_one.
template <int MODEL>
__device__ __forceinline__ void eval_trace_d(const LsParams &a, uint32_t ti, double t0,
                                             double c, double p1, double p2, double m0,
                                             double h0, double shift, double *num,
                                             double &lin, double &den, unsigned &used,
                                             unsigned &nu) {
    const double m = a.mid[ti], h = a.hoff[ti];
    const int w = a.w, tau = a.tau;
    double t;
    if (MODEL == kModelCmp) {
        t = sqrt(t0 * t0 + c * (h * h));
    } else if (MODEL == kModelZocrs) {
        const double dm = m - m0;
        double tmp = t0 + p1 * dm;
        tmp = tmp * tmp + p2 * dm * dm + c * (h * h);
        if (!(tmp >= 0)) return;
        t = sqrt(tmp);
    } else {
        const int ok = oct_time_d(t0, c, p1, m, h, m0, a.apm, h0, &t);
        if (ok < 0) {
            nu++;
            return;
        }
        if (ok == 0) return;
    }
    t = t + shift;
    const double tIndex = t / (double)a.dt;
    // (int) of the reference: truncation toward zero (+inf and NaN land
    // outside the trace)
    const double kf = trunc(tIndex);
    if (!(kf - tau >= 0.0 && kf + tau + 1 < (double)a.S)) return;
    const int k = (int)kf;
    const double frac = tIndex - kf;
    double y1 = amp_at(a, ti, k - tau);
    for (int j = 0; j < w; j++) {
        const double y0 = y1;
        y1 = amp_at(a, ti, k - tau + j + 1);
        const double u = (y1 - y0) * frac + y0;
        num[j] += u;
        lin += u;
        den += u * u;
    }
    used++;
}

__device__ __forceinline__ void reduce_d(const double *num, double lin, double den, int w,
                                         unsigned used, double *sembl, double *stack) {
    *sembl = 0.0;
    *stack = 0.0;
    if (used > 0) {
        double sn = 0.0;
        for (int j = 0; j < w; j++) sn += num[j] * num[j];
        *sembl = sn / ((double)used * den);
        *stack = lin / ((double)used * (double)w);
    }
}

template <int MODEL>
__global__ void __launch_bounds__(kPlainThreads) ls_f64_kernel(LsParams a) {
    const uint32_t mi = blockIdx.x / a.S;
    const uint32_t s = blockIdx.x % a.S;
    if (mi >= a.nM0) return;
    const double m0 = a.m0s[mi];
    const uint32_t first = a.selFirst[mi], cnt = a.selCount[mi];
    const int np = a.np;
    float *out = a.out + (size_t)mi * (2 + np) * a.S;
    if (cnt == 0) {
        if (threadIdx.x < 2 + np) out[(size_t)threadIdx.x * a.S + s] = 0.f;
        return;
    }
    const double t0 = (double)static_cast<float>(s) * (double)a.dt;
    const double h0 = MODEL == kModelOct ? (double)oct_line(a, mi).h0 : 0.0;
    const int w = a.w;
    double best = -1.0, bestStack = 0.0, second = -1.0;
    uint32_t bestP = 0xffffffffu;
    unsigned long long notUsed = 0;

    for (uint32_t p = threadIdx.x; p < a.P; p += blockDim.x) {
        const float *pr = a.params + (size_t)p * np;
        const double c = pr[0];
        const double p1 = np > 1 ? (double)pr[1] : 0.0;
        const double p2 = np > 2 ? (double)pr[2] : 0.0;
        double num[kMaxWindow + 1];
        for (int j = 0; j < w; j++) num[j] = 0.0;
        double lin = 0.0, den = 0.0;
        unsigned used = 0, nu = 0;
        for (uint32_t q = 0; q < cnt; q++)
            eval_trace_d<MODEL>(a, a.selIdx ? a.selIdx[first + q] : first + q, t0, c, p1, p2,
                                m0, h0, 0.0, num, lin, den, used, nu);
        double sembl, stack;
        reduce_d(num, lin, den, w, used, &sembl, &stack);
        // runner-up and argmax (lowest index wins ties, NaN never enters)
        if (sembl > best) {
            second = best;
            best = sembl;
            bestStack = stack;
            bestP = p;
        } else if (sembl > second) {
            second = sembl;
        }
        notUsed += nu;
    }

    __shared__ double shS[kPlainThreads], shK[kPlainThreads], sh2[kPlainThreads];
    __shared__ uint32_t shP[kPlainThreads];
    __shared__ unsigned long long shNu[kPlainThreads];
    shS[threadIdx.x] = best;
    shK[threadIdx.x] = bestStack;
    sh2[threadIdx.x] = second;
    shP[threadIdx.x] = bestP;
    shNu[threadIdx.x] = notUsed;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (uint32_t t = 1; t < blockDim.x; t++) {
            const double os = shS[t];
            const uint32_t op = shP[t];
            if (os > best || (os == best && op < bestP)) {
                second = fmax(best, sh2[t]);
                best = os;
                bestStack = shK[t];
                bestP = op;
            } else {
                second = fmax(second, os);
            }
            notUsed += shNu[t];
        }
        if (a.nearTies && best > 0.0 && second >= 0.0 &&
            best - second <= (double)kNearTieRel * fmax(best, 1e-3))
            atomicAdd(a.nearTies, 1ull);
        out[s] = (float)best;
        out[a.S + s] = (float)bestStack;
        if (bestP != 0xffffffffu) {
            const float *pr = a.params + (size_t)bestP * np;
            out[2 * a.S + s] = 2 / sqrtf(pr[0]);
            for (int j = 1; j < np; j++) out[(size_t)(2 + j) * a.S + s] = pr[j];
        } else {
            for (int j = 0; j < np; j++) out[(size_t)(2 + j) * a.S + s] = 0.f;
        }
        if (MODEL == kModelOct && a.notUsed && notUsed) atomicAdd(a.notUsed + mi, notUsed);
    }
}

// Stretch-free in FP64 (StretchFreeAlgorithm's evaluation with every step in
// FP64): a warp per (midpoint, sample), lanes over n, as sf_kernel.
template <int MODEL>
__global__ void __launch_bounds__(256) sf_f64_kernel(LsParams a, uint32_t nUnits) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int NP = MODEL == kModelCmp ? 1 : (MODEL == kModelZocrs ? 3 : 2);
    const int nn = 2 * a.nmax + 1;
    const uint32_t unit = blockIdx.x * 8 + warp;
    if (unit >= nUnits) return;
    const uint32_t mi = unit / a.S;
    const int s = (int)(unit % a.S);
    const double m0 = a.m0s[mi];
    const uint32_t first = a.selFirst[mi], cnt = a.selCount[mi];
    const float *prior = a.prior + (size_t)mi * NP * a.S;
    const double h0 = MODEL == kModelOct ? (double)oct_line(a, mi).h0 : 0.0;
    double best = -1.0, bestK = 0.0;
    uint32_t bestI = 0xffffffffu;
    unsigned nu = 0;
    for (int ni0 = 0; ni0 < nn; ni0 += 32) {
        const int ni = ni0 + lane;
        const int n = ni - a.nmax;
        const int sn = s - n;
        double sembl = 0.0, stack = 0.0;
        if (ni < nn && sn >= 0 && sn < (int)a.S) {
            const double t0n = (double)static_cast<float>(sn) * (double)a.dt;
            const double v = prior[sn];
            const double c = 4.0 / (v * v);
            const double p1 = MODEL != kModelCmp ? (double)prior[a.S + sn] : 0.0;
            const double p2 = MODEL == kModelZocrs ? (double)prior[2 * a.S + sn] : 0.0;
            double num[kMaxWindow + 1];
            for (int j = 0; j < a.w; j++) num[j] = 0.0;
            double lin = 0.0, den = 0.0;
            unsigned used = 0;
            for (uint32_t q = 0; q < cnt; q++)
                eval_trace_d<MODEL>(a, a.selIdx ? a.selIdx[first + q] : first + q, t0n, c, p1,
                                    p2, m0, h0, (double)n * (double)a.dt, num, lin, den, used,
                                    nu);
            reduce_d(num, lin, den, a.w, used, &sembl, &stack);
        }
        if (ni < nn && sembl > best) {
            best = sembl;
            bestK = stack;
            bestI = (uint32_t)ni;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const double os = __shfl_xor_sync(0xffffffffu, best, o);
        const double ok = __shfl_xor_sync(0xffffffffu, bestK, o);
        const uint32_t oi = __shfl_xor_sync(0xffffffffu, bestI, o);
        if (os > best || (os == best && oi < bestI)) {
            best = os;
            bestK = ok;
            bestI = oi;
        }
        nu += __shfl_xor_sync(0xffffffffu, nu, o);
    }
    if (lane == 0) {
        float *out = a.out + (size_t)mi * 3 * a.S;
        out[s] = (float)best;
        out[a.S + s] = (float)bestK;
        out[2 * a.S + s] = bestI != 0xffffffffu ? (float)((int)bestI - a.nmax) : 0.f;
        if (MODEL == kModelOct && a.notUsed && nu) atomicAdd(a.notUsed + mi, (unsigned long long)nu);
    }
}

cudaError_t launch_sf_f64(const LsParams &p, int model, uint32_t nUnits, cudaStream_t st) {
    if (nUnits == 0) return cudaSuccess;
    const uint32_t grid = (nUnits + 7) / 8;
    if (model == kModelCmp) sf_f64_kernel<kModelCmp><<<grid, 256, 0, st>>>(p, nUnits);
    else if (model == kModelZocrs) sf_f64_kernel<kModelZocrs><<<grid, 256, 0, st>>>(p, nUnits);
    else sf_f64_kernel<kModelOct><<<grid, 256, 0, st>>>(p, nUnits);
    return cudaGetLastError();
}

cudaError_t launch_ls_f64(const LsParams &p, cudaStream_t st) {
    if (p.nM0 == 0 || p.S == 0) return cudaSuccess;
    const uint64_t blocks = (uint64_t)p.nM0 * p.S;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    if (p.np == 1)
        ls_f64_kernel<kModelCmp><<<(unsigned)blocks, kPlainThreads, 0, st>>>(p);
    else if (p.np == 3)
        ls_f64_kernel<kModelZocrs><<<(unsigned)blocks, kPlainThreads, 0, st>>>(p);
    else
        ls_f64_kernel<kModelOct><<<(unsigned)blocks, kPlainThreads, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace hpss
