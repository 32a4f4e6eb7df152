// sf.cu -- stretch-free stack (StretchFreeAlgorithm, common/src/semblance/
// algorithm/StretchFreeAlgorithm.cpp:23-125; kernels cuda/src/semblance/
// kernel/{cmp,zocrs,oct}/stretch_free.cu and common/stretch_free.cu).
//
// For every (midpoint, t0 sample s) and n in [-nmax, nmax] the parameters a
// previous search chose at sample s - n are applied at t0 = (s - n) dt and the
// traveltime is shifted by n dt; the window semblance and stack follow, and
// the n with the highest semblance is kept (strict '>' over n ascending, so
// the most negative n wins ties).  The reference runs only CMP on CUDA (its
// OCT case falls through into `throw`, CudaStretchFreeAlgorithm.cu:86-110);
// all three models run here, with the same per-model traveltime arithmetic
// as the searches.
//
// Three kernels.  sf_block_kernel and sf_batch_kernel (windows 3..11, up to
// 32 n values): a CTA takes 32 consecutive samples of one midpoint, one warp
// per n value and one lane per sample, so a warp's lanes read consecutive
// prior parameters and windows lying side by side in each trace (coalesced
// loads, all lanes busy); the (n, sample) semblances and stacks go to shared
// memory and one warp then scans n upwards for each sample; the batch kernel
// shares each traveltime among the pairs that need it (below).  sf_kernel
// (any window or n count): a warp owns one sample, its lanes the n values.
#include <algorithm>
#include <cstdlib>
#include <cstring>

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
        const OctLine ol = oct_line(a, mi);  // OCT: the midpoint's h0 and factor table
        const float h0 = MODEL == kModelOct ? ol.h0 : 0.f;
        float best = -1.f, bestK = 0.f;
        uint32_t bestI = 0xffffffffu;
        unsigned nu = 0;
        __shared__ float sfBox[kSfWarps][4];  // each warp's displaced-midpoint box (OCT)
        for (int ni0 = 0; ni0 < nn; ni0 += 32) {
            const int ni = ni0 + lane;
            const int n = ni - a.nmax;
            const int sn = s - n;
            const bool member = ni < nn && sn >= 0 && sn < (int)a.S;
            const int snc = member ? sn : s;  // lanes without an evaluation read sample s
            const float t0n = static_cast<float>(snc) * a.dt;
            const float v = prior[snc];
            const float c = 4.0f / (v * v);
            const float p1 = MODEL != kModelCmp ? prior[a.S + snc] : 0.f;
            const float p2 = MODEL == kModelZocrs ? prior[2 * a.S + snc] : 0.f;
            const float nf = static_cast<float>(n);
            // OCT: the (t0, candidate) factors once, the trace factors from
            // the line's table (the same roundings as model_time)
            const OctCand kc = oct_cand(t0n, c, p1, h0);
            float num[kMaxWindow + 1];
            for (int j = 0; j < a.w; j++) num[j] = 0.f;
            float lin = 0.f, den = 0.f;
            unsigned used = 0;
            auto evalTrace = [&](uint32_t ti) {
                float tn;
                int ok;
                if (MODEL == kModelOct) {
                    const float4 tf = __ldg(ol.tab + ti);  // {m, gamma^2, 16h^2h0^2, h^2-h0^2}
                    ok = oct_model_time(kc, tf.y, tf.z, tf.w, t0n, c, p1, tf.x, a.hoff[ti], m0,
                                        a.apm, h0, &tn);
                } else {
                    ok = model_time<MODEL>(t0n, c, p1, p2, a.mid[ti], a.hoff[ti], a.hsq[ti], m0,
                                           a.apm, h0, &tn);
                }
                if (ok < 0) {
                    nu++;
                    return;
                }
                if (ok == 0) return;
                // t_n + n dt as one fused multiply-add, as the reference
                // compiles it (cmp/stretch_free.cu:55)
                const float t = __fmaf_rn(nf, a.dt, tn);
                WinIdx wi = window_index(t, a.dt);
                if (window_in_trace(wi.k, a.tau, (int)a.S)) {
                    const int k0 = wi.k - a.tau;
                    float y1 = amp_at(a, ti, k0);
                    for (int j = 0; j < a.w; j++) {
                        float y0 = y1;
                        y1 = amp_at(a, ti, k0 + j + 1);
                        float u = (y1 - y0) * wi.frac + y0;
                        num[j] += u;
                        lin += u;
                        den += u * u;
                    }
                    used++;
                }
            };
            bool boxOn = false;
            if (MODEL == kModelOct) {
                // the warp's displaced-midpoint box over its lanes' (t0_n,
                // parameters): per block of 32 traces, lane j tests trace j
                // against it and the traces no lane can pass count as not
                // used for every lane without their per-lane test
                const OctWarpBox box = oct_warp_box(a.octBox, member, t0n, p1, kc, h0);
                boxOn = box.on;
                if (boxOn) {
                    oct_box_store(sfBox[warp], box);
                    for (uint32_t qb = 0; qb < cnt; qb += 32) {
                        const uint32_t nb = min(32u, cnt - qb);
                        bool keep = false;
                        if ((uint32_t)lane < nb)
                            keep = oct_box_keep(a, ol, a.selIdx ? a.selIdx[first + qb + lane]
                                                                : first + qb + lane,
                                                sfBox[warp], m0);
                        uint32_t mask = __ballot_sync(0xffffffffu, keep);
                        if (member) nu += nb - (uint32_t)__popc(mask);
                        for (; mask; mask &= mask - 1) {
                            const uint32_t bit = (uint32_t)__ffs(mask) - 1;
                            if (member)
                                evalTrace(a.selIdx ? a.selIdx[first + qb + bit] : first + qb + bit);
                        }
                    }
                }
            }
            if (!boxOn && member)
                for (uint32_t q = 0; q < cnt; q++)
                    evalTrace(a.selIdx ? a.selIdx[first + q] : first + q);
            // an n whose sample s - n lies outside the trace keeps semblance
            // 0 and still takes part in the argmax, as in the reference
            float sembl = 0.f, stack = 0.f;
            if (member) reduce_semblance(num, lin, den, a.w, used, &sembl, &stack);
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
// (selectTracesForOffsetContinuationTrajectory, oct/stretch_free.cu:99-138):
// a trace is used if the parameters chosen at any sample s give a valid
// displaced midpoint within apm at t0 = s dt.  One warp per (midpoint,
// candidate trace) slot over the whole GPU, lanes over the samples, writes a
// 0 / 1 flag into the slot (a.selFirst: the prefix of candCount); the flags
// are then compacted in order (launch_select_compact).
__global__ void sf_select_oct_flags_kernel(LsParams a, const uint32_t *candFirst,
                                           uint64_t total, uint32_t *selIdx) {
    const int lane = threadIdx.x & 31;
    const uint64_t g = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (g >= total) return;  // whole warps
    // the slot's midpoint: the last mi with selFirst[mi] <= g
    uint32_t lo = 0, hi = a.nM0;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if ((uint64_t)a.selFirst[mid] <= g) lo = mid;
        else hi = mid;
    }
    const uint32_t mi = lo;
    const uint32_t ti = candFirst[mi] + (uint32_t)(g - a.selFirst[mi]);
    const float m0 = a.m0s[mi];
    const float h0 = oct_line(a, mi).h0;
    const float *prior = a.prior + (size_t)mi * 2 * a.S;
    const float m = a.mid[ti], h = a.hoff[ti];
    bool used = false;
    for (uint32_t s0 = 0; s0 < a.S && !used; s0 += 32) {
        const uint32_t s = s0 + lane;
        bool hit = false;
        if (s < a.S) {
            const float t0 = static_cast<float>(s) * a.dt;
            const float v = prior[s];
            const float c = 4.0f / (v * v);
            float mh;
            const int e = oct_displaced_midpoint(h, h0, t0, m0, c, prior[a.S + s], &mh);
            hit = e == DE_OK && fabsf(m - mh) <= a.apm;
        }
        used = __any_sync(0xffffffffu, hit);
    }
    if (lane == 0) selIdx[g] = used ? 1u : 0u;
}

// ---------------------------------------------------------------------------
// Block kernels: 32 samples per CTA, warp = n value, lane = sample.
//
// sf_block_kernel (CMP; any model with HPSS_SF_KERNEL=block): each (s, n)
// pair computes its traveltime for every trace.  sf_batch_kernel (ZO-CRS,
// OCT): the traveltime t_n of the pair (s, n) depends on s' = s - n alone
// (the parameters chosen at s' applied at t0 = s' dt); n dt is added
// afterwards.  So the CTA takes its midpoint's traces in batches: first t_n
// and the model's code once per (trace, s') for the 32 + 2 nmax samples s'
// its pairs reach, into shared memory (phase 1, all threads over the batch's
// (trace, s') items), then every (s, n) pair walks the batch's traces in
// order with t_n from there (phase 2): 32 + 2 nmax traveltimes per trace
// instead of 32 (2 nmax + 1) (OCT 8 midpoints x 3 h0: 63.2 -> 46.7 ms;
// ZO-CRS 16 midpoints: 3.58 -> 3.37 ms).  CMP, whose traveltime is one fused
// multiply-add and a square root, stays with the per-pair form (the two
// phases and their barriers cost it 3-9 %).  In both kernels each pair's sums
// take the same values in the same trace order as the warp kernel's, so the
// blocks are the same bit for bit; the OCT pairs count a trace as not used
// where its code says so, which is where the warp kernel's box test or
// per-lane test does.
constexpr int kSfBlockMaxN = 32;                  // n values (warps) per CTA
constexpr int kSfSlots = 32 + kSfBlockMaxN - 1;   // s' = s - n: 32 + 2 nmax <= 63
constexpr int kSfBatch = 64;                      // traces per batch

template <int MODEL, int W>
__global__ void __maxnreg__(40)
sf_block_kernel(LsParams a, uint32_t blocksPerM0, uint32_t nUnits) {
    __shared__ float pairS[kSfBlockMaxN][32], pairK[kSfBlockMaxN][32];  // [n][sample]
    __shared__ float sfBox[kSfBlockMaxN][4];  // each warp's displaced-midpoint box (OCT)
    constexpr int NP = MODEL == kModelCmp ? 1 : (MODEL == kModelZocrs ? 3 : 2);
    const int lane = threadIdx.x & 31;
    const int ni = threadIdx.x >> 5;  // this warp's n value: n = ni - nmax
    const int S = (int)a.S;
    const int nn = 2 * a.nmax + 1;    // = warps of the CTA
    for (uint32_t unit = blockIdx.x; unit < nUnits; unit += gridDim.x) {
        const uint32_t mi = unit / blocksPerM0;
        const int s = (int)(unit % blocksPerM0) * 32 + lane;
        const float m0 = a.m0s[mi];
        const uint32_t first = a.selFirst[mi], cnt = a.selCount[mi];
        const float *prior = a.prior + (size_t)mi * NP * a.S;
        const OctLine ol = oct_line(a, mi);  // OCT: the midpoint's h0 and factor table
        const float h0 = MODEL == kModelOct ? ol.h0 : 0.f;
        unsigned nu = 0;
        const int n = ni - a.nmax;
        const int sn = s - n;
        const bool member = s < S && sn >= 0 && sn < S;
        const int snc = member ? sn : min(s, S - 1);  // a valid sample for the others
        const float t0n = static_cast<float>(snc) * a.dt;
        const float v = prior[snc];
        const float c = 4.0f / (v * v);
        const float p1 = MODEL != kModelCmp ? prior[a.S + snc] : 0.f;
        const float p2 = MODEL == kModelZocrs ? prior[2 * a.S + snc] : 0.f;
        const float nf = static_cast<float>(n);
        const OctCand kc = oct_cand(t0n, c, p1, h0);
        float num[W];
#pragma unroll
        for (int j = 0; j < W; j++) num[j] = 0.f;
        float lin = 0.f, den = 0.f;
        unsigned used = 0;
        auto evalTrace = [&](uint32_t ti) {
            float tn;
            int ok;
            if (MODEL == kModelOct) {
                const float4 tf = __ldg(ol.tab + ti);  // {m, gamma^2, 16h^2h0^2, h^2-h0^2}
                ok = oct_model_time(kc, tf.y, tf.z, tf.w, t0n, c, p1, tf.x, a.hoff[ti], m0,
                                    a.apm, h0, &tn);
            } else {
                ok = model_time<MODEL>(t0n, c, p1, p2, a.mid[ti], a.hoff[ti], a.hsq[ti], m0,
                                       a.apm, h0, &tn);
            }
            if (ok < 0) {
                nu++;
                return;
            }
            if (ok == 0) return;
            // t_n + n dt as one fused multiply-add (cmp/stretch_free.cu:55)
            const float t = __fmaf_rn(nf, a.dt, tn);
            const WinIdx wi = window_index(t, a.dt);
            if (window_in_trace(wi.k, a.tau, S)) {
                accum_window<W>(a, ti, wi.k - a.tau, wi.frac, num, lin, den);
                used++;
            }
        };
        bool boxOn = false;
        if (MODEL == kModelOct) {
            // the warp's displaced-midpoint box over its lanes' (t0_n,
            // parameters); traces no lane can pass count as not used for
            // every member lane without their per-lane test
            const OctWarpBox box = oct_warp_box(a.octBox, member, t0n, p1, kc, h0);
            boxOn = box.on;
            if (boxOn) {
                oct_box_store(sfBox[ni], box);
                for (uint32_t qb = 0; qb < cnt; qb += 32) {
                    const uint32_t nb = min(32u, cnt - qb);
                    bool keep = false;
                    if ((uint32_t)lane < nb)
                        keep = oct_box_keep(a, ol, a.selIdx ? a.selIdx[first + qb + lane]
                                                            : first + qb + lane,
                                            sfBox[ni], m0);
                    uint32_t mask = __ballot_sync(0xffffffffu, keep);
                    if (member) nu += nb - (uint32_t)__popc(mask);
                    for (; mask; mask &= mask - 1) {
                        const uint32_t bit = (uint32_t)__ffs(mask) - 1;
                        if (member)
                            evalTrace(a.selIdx ? a.selIdx[first + qb + bit] : first + qb + bit);
                    }
                }
            }
        }
        if (!boxOn && member)
            for (uint32_t q = 0; q < cnt; q++) evalTrace(a.selIdx ? a.selIdx[first + q] : first + q);
        // an n whose sample s - n lies outside the trace keeps semblance 0 and
        // still takes part in the argmax, as in the reference
        float sembl = 0.f, stack = 0.f;
        if (member) reduce_semblance(num, lin, den, W, used, &sembl, &stack);
        pairS[ni][lane] = sembl;
        pairK[ni][lane] = stack;
        if (MODEL == kModelOct && a.notUsed) {
#pragma unroll
            for (int o = 16; o; o >>= 1) nu += __shfl_xor_sync(0xffffffffu, nu, o);
            if (lane == 0 && nu) atomicAdd(a.notUsed + mi, (unsigned long long)nu);
        }
        __syncthreads();
        // per sample: strict '>' over n ascending (the most negative n wins ties)
        if (ni == 0 && s < S) {
            float best = -1.f, bestK = 0.f;
            int bestI = -1;
            for (int k = 0; k < nn; k++) {
                const float sv = pairS[k][lane];
                if (sv > best) {
                    best = sv;
                    bestK = pairK[k][lane];
                    bestI = k;
                }
            }
            float *out = a.out + (size_t)mi * 3 * a.S;
            out[s] = best;
            out[a.S + s] = bestK;
            out[2 * a.S + s] = bestI >= 0 ? (float)(bestI - a.nmax) : 0.f;
        }
        __syncthreads();  // the pair arrays are read before the next unit writes them
    }
}

template <int MODEL, int W>
__global__ void __maxnreg__(40)
sf_batch_kernel(LsParams a, uint32_t blocksPerM0, uint32_t nUnits) {
    static_assert(MODEL != kModelCmp, "CMP takes sf_block_kernel");
    __shared__ float pairS[kSfBlockMaxN][32], pairK[kSfBlockMaxN][32];  // [n][sample]
    // t_n and model_time's code per (trace of the batch, s'), the batch's
    // trace indices; per s' slot t0, c = 4 / v^2, the other parameters and
    // (OCT) the candidate factors
    __shared__ float tnS[kSfBatch][kSfSlots + 1];
    __shared__ signed char codeS[kSfBatch][kSfSlots + 1];
    __shared__ uint32_t tiS[kSfBatch];
    __shared__ float slotT0[kSfSlots], slotC[kSfSlots], slotP1[kSfSlots], slotP2[kSfSlots];
    __shared__ OctCand slotK[MODEL == kModelOct ? kSfSlots : 1];
    constexpr int NP = MODEL == kModelCmp ? 1 : (MODEL == kModelZocrs ? 3 : 2);
    const int lane = threadIdx.x & 31;
    const int ni = threadIdx.x >> 5;  // this warp's n value: n = ni - nmax
    const int S = (int)a.S;
    const int nn = 2 * a.nmax + 1;    // = warps of the CTA
    const int nSlots = 32 + 2 * a.nmax;
    for (uint32_t unit = blockIdx.x; unit < nUnits; unit += gridDim.x) {
        const uint32_t mi = unit / blocksPerM0;
        const int s0 = (int)(unit % blocksPerM0) * 32;
        const int s = s0 + lane;
        const float m0 = a.m0s[mi];
        const uint32_t first = a.selFirst[mi], cnt = a.selCount[mi];
        const float *prior = a.prior + (size_t)mi * NP * a.S;
        const OctLine ol = oct_line(a, mi);  // OCT: the midpoint's h0 and factor table
        const float h0 = MODEL == kModelOct ? ol.h0 : 0.f;
        // slot i holds s' = s0 - nmax + i (slots outside the trace serve no pair)
        if ((int)threadIdx.x < nSlots) {
            const int sp = s0 - a.nmax + (int)threadIdx.x;
            const int spc = min(max(sp, 0), S - 1);
            const float t0n = static_cast<float>(spc) * a.dt;
            const float v = prior[spc];
            const float c = 4.0f / (v * v);
            const float p1 = MODEL != kModelCmp ? prior[a.S + spc] : 0.f;
            slotT0[threadIdx.x] = t0n;
            slotC[threadIdx.x] = c;
            slotP1[threadIdx.x] = p1;
            slotP2[threadIdx.x] = MODEL == kModelZocrs ? prior[2 * a.S + spc] : 0.f;
            if constexpr (MODEL == kModelOct) slotK[threadIdx.x] = oct_cand(t0n, c, p1, h0);
        }
        unsigned nu = 0;
        const int n = ni - a.nmax;
        const bool member = s < S && s - n >= 0 && s - n < S;
        const int slot = lane + a.nmax - n;  // s' = s - n
        const float nf = static_cast<float>(n);
        float num[W];
#pragma unroll
        for (int j = 0; j < W; j++) num[j] = 0.f;
        float lin = 0.f, den = 0.f;
        unsigned used = 0;
        for (uint32_t qb = 0; qb < cnt; qb += kSfBatch) {
            const int nb = (int)min((uint32_t)kSfBatch, cnt - qb);
            __syncthreads();  // slots written; the previous batch is consumed
            // phase 1: t_n and the code of every (trace, s') of the batch
            for (int item = (int)threadIdx.x; item < nb * nSlots; item += (int)blockDim.x) {
                const int j = item / nSlots, i = item - j * nSlots;
                const uint32_t ti = a.selIdx ? a.selIdx[first + qb + j] : first + qb + j;
                const int sp = s0 - a.nmax + i;
                float tn = 0.f;
                int ok = 0;
                if (sp >= 0 && sp < S) {
                    if constexpr (MODEL == kModelOct) {
                        const float4 tf = __ldg(ol.tab + ti);  // {m, gamma^2, 16h^2h0^2, h^2-h0^2}
                        ok = oct_model_time(slotK[i], tf.y, tf.z, tf.w, slotT0[i], slotC[i],
                                            slotP1[i], tf.x, a.hoff[ti], m0, a.apm, h0, &tn);
                    } else {
                        ok = model_time<MODEL>(slotT0[i], slotC[i], slotP1[i], slotP2[i],
                                               a.mid[ti], a.hoff[ti], a.hsq[ti], m0, a.apm, h0,
                                               &tn);
                    }
                }
                tnS[j][i] = tn;
                codeS[j][i] = (signed char)ok;
                if (i == 0) tiS[j] = ti;
            }
            __syncthreads();
            // phase 2: this pair over the batch's traces, in order
            if (member) {
                for (int j = 0; j < nb; j++) {
                    const int ok = codeS[j][slot];
                    if (ok < 0) {
                        nu++;
                        continue;
                    }
                    if (ok == 0) continue;
                    // t_n + n dt as one fused multiply-add (cmp/stretch_free.cu:55)
                    const float t = __fmaf_rn(nf, a.dt, tnS[j][slot]);
                    const WinIdx wi = window_index(t, a.dt);
                    if (window_in_trace(wi.k, a.tau, S)) {
                        accum_window<W>(a, tiS[j], wi.k - a.tau, wi.frac, num, lin, den);
                        used++;
                    }
                }
            }
        }
        // an n whose sample s - n lies outside the trace keeps semblance 0 and
        // still takes part in the argmax, as in the reference
        float sembl = 0.f, stack = 0.f;
        if (member) reduce_semblance(num, lin, den, W, used, &sembl, &stack);
        pairS[ni][lane] = sembl;
        pairK[ni][lane] = stack;
        if (MODEL == kModelOct && a.notUsed) {
#pragma unroll
            for (int o = 16; o; o >>= 1) nu += __shfl_xor_sync(0xffffffffu, nu, o);
            if (lane == 0 && nu) atomicAdd(a.notUsed + mi, (unsigned long long)nu);
        }
        __syncthreads();
        // per sample: strict '>' over n ascending (the most negative n wins ties)
        if (ni == 0 && s < S) {
            float best = -1.f, bestK = 0.f;
            int bestI = -1;
            for (int k = 0; k < nn; k++) {
                const float sv = pairS[k][lane];
                if (sv > best) {
                    best = sv;
                    bestK = pairK[k][lane];
                    bestI = k;
                }
            }
            float *out = a.out + (size_t)mi * 3 * a.S;
            out[s] = best;
            out[a.S + s] = bestK;
            out[2 * a.S + s] = bestI >= 0 ? (float)(bestI - a.nmax) : 0.f;
        }
        __syncthreads();  // the pair arrays and slots are read before the next unit writes them
    }
}

template <typename K>
static cudaError_t launch_sf_blocks(K kernel, const LsParams &p, int numSms, cudaStream_t st) {
    const uint32_t blocksPerM0 = (p.S + 31) / 32;
    const uint64_t units = (uint64_t)p.nM0 * blocksPerM0;
    if (units > 0xffffffffull) return cudaErrorInvalidConfiguration;
    const int threads = (2 * p.nmax + 1) * 32;
    int perSm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, threads, 0);
    if (e != cudaSuccess) return e;
    const uint32_t grid =
        (uint32_t)std::min<uint64_t>(units, (uint64_t)numSms * (uint64_t)std::max(perSm, 1));
    kernel<<<grid, threads, 0, st>>>(p, blocksPerM0, (uint32_t)units);
    return cudaGetLastError();
}

template <int MODEL, int W>
static cudaError_t launch_sf_block(const LsParams &p, int numSms, bool perPair, cudaStream_t st) {
    if constexpr (MODEL == kModelCmp) {
        return launch_sf_blocks(sf_block_kernel<MODEL, W>, p, numSms, st);
    } else {
        return perPair ? launch_sf_blocks(sf_block_kernel<MODEL, W>, p, numSms, st)
                       : launch_sf_blocks(sf_batch_kernel<MODEL, W>, p, numSms, st);
    }
}

template <int MODEL>
static cudaError_t launch_sf_model(const LsParams &p, int numSms, cudaStream_t st) {
    const int nn = 2 * p.nmax + 1;
    // HPSS_SF_KERNEL=warp: the warp-per-sample kernel for every call;
    // =block: the per-pair block kernel for every model (the kernels give the
    // same results bit for bit)
    const char *pick = std::getenv("HPSS_SF_KERNEL");
    const bool warpKernel = pick && std::strcmp(pick, "warp") == 0;
    const bool perPair = pick && std::strcmp(pick, "block") == 0;
    if (nn <= kSfBlockMaxN && !warpKernel) {
        switch (p.w) {
            case 3: return launch_sf_block<MODEL, 3>(p, numSms, perPair, st);
            case 5: return launch_sf_block<MODEL, 5>(p, numSms, perPair, st);
            case 7: return launch_sf_block<MODEL, 7>(p, numSms, perPair, st);
            case 9: return launch_sf_block<MODEL, 9>(p, numSms, perPair, st);
            case 11: return launch_sf_block<MODEL, 11>(p, numSms, perPair, st);
            default: break;
        }
    }
    const uint64_t units = (uint64_t)p.nM0 * p.S;
    if (units > 0xffffffffull) return cudaErrorInvalidConfiguration;
    const uint32_t grid = (uint32_t)std::min<uint64_t>((units + kSfWarps - 1) / kSfWarps,
                                                       (uint64_t)numSms * 8);
    sf_kernel<MODEL><<<grid, kSfWarps * 32, 0, st>>>(p, (uint32_t)units);
    return cudaGetLastError();
}

cudaError_t launch_sf(const LsParams &p, int model, int numSms, cudaStream_t st) {
    if (p.nM0 == 0 || p.S == 0) return cudaSuccess;
    if (model == kModelCmp) return launch_sf_model<kModelCmp>(p, numSms, st);
    if (model == kModelZocrs) return launch_sf_model<kModelZocrs>(p, numSms, st);
    return launch_sf_model<kModelOct>(p, numSms, st);
}

cudaError_t launch_sf_select_oct(const LsParams &p, const uint32_t *candFirst,
                                 const uint32_t *candCount, uint32_t *selIdx,
                                 uint32_t *selCount, uint64_t total, cudaStream_t st) {
    if (p.nM0 == 0) return cudaSuccess;
    if (total > 0) {
        const uint64_t blocks = (total * 32 + 255) / 256;
        if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
        sf_select_oct_flags_kernel<<<(uint32_t)blocks, 256, 0, st>>>(p, candFirst, total, selIdx);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return launch_select_compact(p, candFirst, candCount, selIdx, selCount, st);
}

}  // namespace hpss
