// ls_tuned.cuh -- the tuned linear-search kernel for the CMP and ZO-CRS
// traveltimes (template; instantiated in ls_tuned_{cmp,zocrs}{,_exact}.cu so
// they compile in parallel; the OCT kernel is ls_oct.cu).
//
// Work unit: one midpoint x 32 consecutive t0 samples (lane = sample).  The
// 8 warps of a CTA split the candidates; candidates are visited in chunks of
// 8*R (R per thread, independent accumulators for ILP).  For every chunk the
// CTA computes, per selected trace, the sample span any window of that chunk
// and tile can touch (monotone / interval bounds of the traveltime over the
// tile's t0 range and the chunk's parameter box), stages those spans into
// shared memory, and evaluates all (sample, candidate) pairs of the chunk
// against them.  Lanes of a warp read nearly consecutive shared-memory words
// (one sample apart), so the window loads are free of bank conflicts.  The
// per-candidate arithmetic is the reference's (interface.h:26-55), so the
// semblances and chosen candidates equal the plain kernel's bit for bit (the
// stack too, except where the pair kernel derives the linear sum from the
// per-tap sums, see EXACT_STACK below).  The argmax over candidates
// is kept in registers and reduced across warps at the end (lowest index wins
// ties).  CTAs are persistent over the work units; a call with more units
// than resident CTAs hands them out from an atomic counter, the midpoints
// ordered by descending selected traces, so that the heaviest units start
// first and no CTA idles while others finish.  A call with few
// midpoints has too few (midpoint, tile) units to fill the GPU (one CMP
// midpoint of 2000 samples: 63 units for 2-3 CTAs on each of 152 SMs); the
// host then splits the candidate chunks into `parts` contiguous ranges, a unit
// becomes (midpoint, tile, part), and the ordered merge of ls_oct.cu combines
// the parts (lowest candidate index still wins ties).
#pragma once

#include <cuda_fp16.h>

#include <type_traits>

#include "hpss_device.cuh"
#include "hpss_internal.h"
#include "stage.cuh"

namespace hpss {

// ---------------------------------------------------------------------------
// Branch-free variant for the CMP and ZO-CRS models.
//
// Per trace, the window position of every candidate of the thread is computed
// first (independent chains); a window outside the trace is redirected to a
// zero pad at the start of shared memory, so it adds exactly 0 to every sum
// and is not counted in `used` -- the same sums as the reference's skip.
// The window arithmetic runs on candidate pairs with Blackwell's packed
// f32x2 FMA / ADD (per lane the same IEEE operation as the scalar form), so a
// warp instruction advances two candidates.
// ---------------------------------------------------------------------------
constexpr int kZeroPad = 32;  // floats of zeros before the staged spans

struct __align__(16) TraceMeta2 {
    int base;   // shared-memory index of sample 0 of the trace
    float hsq;  // h * h
    float dm;   // m - m0 (ZO-CRS)
    int len;    // staged samples | kFullTrace when every window is in the trace
};
constexpr int kFullTrace = int(0x80000000u);
constexpr int kLenMask = 0x7fffffff;

// stage size per CTA for MINB resident CTAs per SM
template <int MINB>
struct Stage2 {
    static constexpr int kFloats = MINB >= 3 ? 16384 : 24576;
};

template <int MINB>
struct Tuned2Smem {
    float y[Stage2<MINB>::kFloats];
    TraceMeta2 meta[kTunedThreads];
    int lo[kTunedThreads];
    int ti[kTunedThreads];
    int warpSum[kTunedWarps];
    int warpKeep[kTunedWarps];
    int warpLen[kTunedWarps];  // staged floats of the warp's kept traces
    float bestS[kTunedWarps][kTileSamples];
    float bestK[kTunedWarps][kTileSamples];
    uint32_t bestP[kTunedWarps][kTileSamples];
    float bestSec[kTunedWarps][kTileSamples];
    unsigned long long stageBar;  // mbarrier of the bulk copies of a staging round
    uint32_t nextUnit;            // work-queue unit handed to the CTA
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }


// EXACT_STACK: accumulate the linear sum tap by tap in the reference's order
// (stack bit-identical to the reference); otherwise the linear sum is taken
// as the sum of the W per-tap numerator sums at the end (the same quantity
// summed in another order: one FADD2 per tap less, the stack within a few
// ulp).  Semblance and the chosen candidate are identical either way.
//
// PREC: precision modes (HPSS_PREC_*; 0 = the reference's FP32 arithmetic).
//  * kPrecTt64 (ZO-CRS): the squared time in FP64, the time rounded to FP32
//    once (zocrs_time_tt64, the plain kernel's form: same bits);
//  * kPrecCompensated: when window x selected traces exceeds 4096 terms, the
//    window sums are compensated across staging rounds: each round (the
//    traces one stage holds, at most 256) is summed in FP32 as usual, and
//    the round's sums are added into running totals with Knuth's two-sum,
//    their rounding errors kept in compensation terms and added once at the
//    end.  The error is then that of one round's plain sum instead of the
//    whole aperture's.
//
// S16: 16-bit rows staged by the TMA engine.  Spans are rounded to 8 samples
// (16 bytes of 16-bit data); each kept trace's raw span is bulk-copied into
// the upper half of its FP32 area of the stage and widened in place, a warp
// per trace, in chunks of 128 samples taken in increasing order: a chunk's
// lanes read all their raw words before any writes, and the FP32 words of
// element i only overwrite raw elements below i, which earlier chunks have
// read.  The widened values are those of the S16 = false kernel's LSU
// widening (which also serves the precision modes and the exact stack).
template <int MODEL, int W, int NP, int MINB, bool EXACT_STACK, int PREC = 0, bool S16 = false>
__global__ void __launch_bounds__(kTunedThreads, MINB)
ls_tuned2_kernel(LsParams a, uint32_t tiles, uint32_t nUnits) {
    constexpr bool TT64 = (PREC & kPrecTt64) != 0 && MODEL == kModelZocrs;
    constexpr bool COMP = (PREC & kPrecCompensated) != 0;
    constexpr int kStage = Stage2<MINB>::kFloats;
    constexpr int R = 2 * NP;
    extern __shared__ __align__(16) unsigned char smemRaw[];
    Tuned2Smem<MINB> &sm = *reinterpret_cast<Tuned2Smem<MINB> *>(smemRaw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int np = a.np;
    const int S = (int)a.S, tau = a.tau;
    const float2 kNeg1 = f2(-1.f, -1.f);
    constexpr int kLastBase = kStage - W - 1;
    // window starts k - tau that keep the whole window inside the trace
    const unsigned winSpan = S > 2 * tau + 1 ? (unsigned)(S - 2 * tau - 1) : 0u;
    const float rdt = 1.0f / a.dt;
    const float2 rdt2 = f2(rdt, rdt);
    const float2 kMagic2 = f2(8388608.f, 8388608.f);      // 2^23
    const float2 kNegMagic2 = f2(-8388608.f, -8388608.f);
    const int magicTau = 0x4B000000 + tau;                  // bits of 2^23, plus tau

#ifdef HPSS_CHECKED
    const uint32_t drillBytes = a.stageDrillBytes;
#else
    constexpr uint32_t drillBytes = 0;
#endif
    // polls of the staging barrier before a round counts as timed out (the
    // timeout drill of checked builds gives up sooner)
    const uint32_t waitLimit = drillBytes ? (1u << 12) : (1u << 22);

    if (threadIdx.x < kZeroPad) sm.y[threadIdx.x] = 0.f;
    if (threadIdx.x == 0) stage_bar_init(&sm.stageBar);
    __syncthreads();
    uint32_t stagePhase = 0;  // parity of the staging barrier's current phase

    for (uint32_t unit = blockIdx.x;; unit += gridDim.x) {
        // work queue: the next unit for this CTA (heaviest midpoints first
        // when the host ordered them), else static round-robin
        if (a.unitCounter) {
            __syncthreads();  // every thread has read the previous unit
            if (threadIdx.x == 0) sm.nextUnit = atomicAdd(a.unitCounter, 1u);
            __syncthreads();
            unit = sm.nextUnit;
        }
        if (unit >= nUnits) break;
        // unit = (midpoint, tile, candidate part), part fastest
        const uint32_t part = unit % a.parts;
        const uint32_t mt = unit / a.parts;
        const uint32_t mi = a.order ? a.order[mt / tiles] : mt / tiles;
        const int s0 = (int)(mt % tiles) * kTileSamples;
        const int s = s0 + lane;
        const int sc = min(s, S - 1);
        const float t0 = static_cast<float>(sc) * a.dt;
        const float t0sq = __fmul_rn(t0, t0);
        const float2 t0sq2 = f2(t0sq, t0sq), t0p2 = f2(t0, t0);
        const float t0a = static_cast<float>(s0) * a.dt;
        const float t0b = static_cast<float>(min(s0 + kTileSamples - 1, S - 1)) * a.dt;
        const float m0 = a.m0s[mi];
        const uint32_t first = a.selFirst[mi], cnt = a.selCount[mi];
        float *out = a.out + (size_t)mi * (2 + np) * a.S;

        if (cnt == 0) {
            // split calls: the merge writes the zero block
            if (a.parts == 1 && warp < 2 + np && s < S) out[(size_t)warp * a.S + s] = 0.f;
            continue;
        }

        float best = -1.f, bestStack = 0.f;
        uint32_t bestP = 0xffffffffu;
        float second = -1.f;  // runner-up semblance (near-tie count)

        const uint32_t chunkEnd =
            a.parts == 1 ? a.nChunks : min((part + 1) * a.chunksPerPart, a.nChunks);
        for (uint32_t chunk = part * a.chunksPerPart; chunk < chunkEnd; chunk++) {
            float cc[R], c1[R], c2[R];
            bool valid[R];
#pragma unroll
            for (int r = 0; r < R; r++) {
                uint32_t p = chunk * a.chunkSize + warp * R + r;
                valid[r] = p < a.P;
                uint32_t pc = valid[r] ? p : a.P - 1;
                const float *pr = a.params + (size_t)pc * np;
                cc[r] = pr[0];
                c1[r] = MODEL == kModelZocrs ? pr[1] : 0.f;
                c2[r] = MODEL == kModelZocrs ? pr[2] : 0.f;
            }
            const float *cb = a.chunkBounds + (size_t)chunk * 2 * np;
            float cbl[6];
#pragma unroll
            for (int j = 0; j < 6; j++) cbl[j] = j < 2 * np ? cb[j] : 0.f;

            float2 num[NP][W], lin[NP], den[NP];
            unsigned used[R];
            unsigned usedFull = 0;  // traces evaluated on the FULL path
#pragma unroll
            for (int q = 0; q < NP; q++) {
#pragma unroll
                for (int j = 0; j < W; j++) num[q][j] = f2(0.f, 0.f);
                lin[q] = den[q] = f2(0.f, 0.f);
            }
            // compensated sums: running totals and compensations over the
            // staging rounds (COMP, more than 4096 window x trace terms)
            const bool comp = COMP && (uint64_t)W * cnt > 4096u;
            float2 numT[COMP ? NP : 1][COMP ? W : 1], numC[COMP ? NP : 1][COMP ? W : 1];
            float2 linT[COMP ? NP : 1], linC[COMP ? NP : 1], denT[COMP ? NP : 1],
                denC[COMP ? NP : 1];
            if constexpr (COMP) {
#pragma unroll
                for (int q = 0; q < NP; q++) {
#pragma unroll
                    for (int j = 0; j < W; j++) numT[q][j] = numC[q][j] = f2(0.f, 0.f);
                    linT[q] = linC[q] = denT[q] = denC[q] = f2(0.f, 0.f);
                }
            }
#pragma unroll
            for (int r = 0; r < R; r++) used[r] = 0;

            for (uint32_t q0 = 0; q0 < cnt;) {
                __syncthreads();
                const uint32_t q = q0 + threadIdx.x;
                int lo = 0, len = 0;
                float tm = 0.f, thsq = 0.f;
                bool full = false;
                if (q < cnt) {
                    const uint32_t ti = a.selIdx ? a.selIdx[first + q] : first + q;
                    tm = a.mid[ti];
                    thsq = a.hsq[ti];
                    trace_span<MODEL, S16 ? 8 : 4>(a, cbl, m0, t0a, t0b, tm, thsq, &lo, &len,
                                                   &full);
                }
                int incl = len;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int v = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += v;
                }
                if (lane == 31) sm.warpSum[warp] = incl;
                __syncthreads();
                int woff = kZeroPad;
#pragma unroll
                for (int wv = 0; wv < kTunedWarps; wv++)
                    woff += wv < warp ? sm.warpSum[wv] : 0;
                const int off = woff + incl - len;
                const bool fits = (q < cnt) && (off + len <= kStage);
                // traces whose span is empty contribute nothing: compact the
                // others so the evaluation loop has no per-trace branch
                const bool keep = fits && len > 0;
                const unsigned keepMask = __ballot_sync(0xffffffffu, keep);
                const int keptLen = __reduce_add_sync(0xffffffffu, keep ? len : 0);
                if (lane == 0) {
                    sm.warpKeep[warp] = __popc(keepMask);
                    sm.warpLen[warp] = keptLen;
                }
                const int nfit = __syncthreads_count(fits);
                int slot = __popc(keepMask & ((1u << lane) - 1u));
#pragma unroll
                for (int wv = 0; wv < kTunedWarps; wv++) slot += wv < warp ? sm.warpKeep[wv] : 0;
                int nkeep = 0;
#pragma unroll
                for (int wv = 0; wv < kTunedWarps; wv++) nkeep += sm.warpKeep[wv];
                if (keep) {
                    TraceMeta2 md;
                    md.base = off - lo;
                    md.hsq = thsq;
                    md.dm = tm - m0;
                    md.len = len | (full ? kFullTrace : 0);
                    sm.meta[slot] = md;
                    sm.lo[slot] = lo;
                    sm.ti[slot] = (int)(a.selIdx ? a.selIdx[first + q] : first + q);
                }
                if (nfit == 0) {
                    if (threadIdx.x == 0) atomicOr(a.errorWord, kErrSpanOverflow);
                    break;
                }
                __syncthreads();
                if constexpr (S16) {
                    // 16-bit rows: one bulk copy of the raw span into the
                    // upper half of the trace's FP32 area, then widened in place
                    if (threadIdx.x == 0) {
                        uint32_t floats = 0;
#pragma unroll
                        for (int wv = 0; wv < kTunedWarps; wv++) floats += (uint32_t)sm.warpLen[wv];
                        stage_bar_expect(&sm.stageBar, floats * 2u + drillBytes);
                    }
                    if (keep) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        const uint32_t ti = a.selIdx ? a.selIdx[first + q] : first + q;
                        stage_bulk_copy(reinterpret_cast<uint16_t *>(sm.y + off) + len,
                                        a.samples16 + (size_t)ti * a.stride + lo, (uint32_t)len * 2u,
                                        &sm.stageBar);
                    }
                    const bool ok = stage_bar_wait(&sm.stageBar, stagePhase, waitLimit);
                    stagePhase ^= 1u;
                    if (__syncthreads_or(!ok)) {
                        if (threadIdx.x == 0) atomicOr(a.errorWord, kErrTimeout);
                        stage_bar_wait(&sm.stageBar, stagePhase ^ 1u, waitLimit);
                        return;
                    }
                    for (int j = warp; j < nkeep; j += kTunedWarps) {
                        const TraceMeta2 md = sm.meta[j];
                        const int lo_j = sm.lo[j];
                        const int n16 = md.len & kLenMask;
                        float *dst = sm.y + md.base + lo_j;
                        const uint16_t *raw = reinterpret_cast<const uint16_t *>(dst) + n16;
                        const float sc = a.storage == 2 ? a.scale[sm.ti[j]] : 1.f;
                        for (int c0 = 0; c0 < n16; c0 += 128) {
                            const int i = c0 + 4 * lane;
                            uint2 r4 = make_uint2(0u, 0u);
                            if (i < n16) r4 = *reinterpret_cast<const uint2 *>(raw + i);
                            __syncwarp();  // every raw word of the chunk read before any write
                            if (i < n16) {
                                *reinterpret_cast<float4 *>(dst + i) =
                                    a.storage == 2
                                        ? make_float4(half_bits_to_float(r4.x & 0xffffu) * sc,
                                                      half_bits_to_float(r4.x >> 16) * sc,
                                                      half_bits_to_float(r4.y & 0xffffu) * sc,
                                                      half_bits_to_float(r4.y >> 16) * sc)
                                        : make_float4(__uint_as_float(r4.x << 16),
                                                      __uint_as_float(r4.x & 0xffff0000u),
                                                      __uint_as_float(r4.y << 16),
                                                      __uint_as_float(r4.y & 0xffff0000u));
                            }
                        }
                    }
                } else {
                if (a.samples16 == nullptr) {
                    // FP32: one bulk copy per span on the TMA engine, the
                    // round's bytes counted off the staging barrier
                    if (threadIdx.x == 0) {
                        uint32_t floats = 0;
#pragma unroll
                        for (int wv = 0; wv < kTunedWarps; wv++) floats += (uint32_t)sm.warpLen[wv];
                        stage_bar_expect(&sm.stageBar, floats * 4u + drillBytes);
                    }
                    if (keep) {
                        // the previous round's reads of the stage are ordered
                        // before the async-proxy writes
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        const uint32_t ti = a.selIdx ? a.selIdx[first + q] : first + q;
                        stage_bulk_copy(sm.y + off, a.samples + (size_t)ti * a.stride + lo,
                                        (uint32_t)len * 4u, &sm.stageBar);
                    }
                    const bool ok = stage_bar_wait(&sm.stageBar, stagePhase, waitLimit);
                    stagePhase ^= 1u;
                    if (__syncthreads_or(!ok)) {
                        // copies did not complete in time: report, wait (again
                        // bounded) for this CTA's copies in flight, and leave
                        if (threadIdx.x == 0) atomicOr(a.errorWord, kErrTimeout);
                        stage_bar_wait(&sm.stageBar, stagePhase ^ 1u, waitLimit);
                        return;
                    }
                }
                for (int j = warp; j < nkeep && a.samples16 != nullptr; j += kTunedWarps) {
                    const TraceMeta2 md = sm.meta[j];
                    const int lo_j = sm.lo[j];
                    float4 *dst = reinterpret_cast<float4 *>(sm.y + md.base + lo_j);
                    {
                        // 16-bit storage: 4 samples per 8-byte load, widened to FP32
                        const uint2 *src = reinterpret_cast<const uint2 *>(
                            a.samples16 + (size_t)sm.ti[j] * a.stride + lo_j);
                        const float sc = a.storage == 2 ? a.scale[sm.ti[j]] : 1.f;
                        for (int v = lane; v < ((md.len & kLenMask) >> 2); v += 32) {
                            const uint2 q = __ldg(src + v);
                            dst[v] = a.storage == 2
                                         ? make_float4(half_bits_to_float(q.x & 0xffffu) * sc,
                                                       half_bits_to_float(q.x >> 16) * sc,
                                                       half_bits_to_float(q.y & 0xffffu) * sc,
                                                       half_bits_to_float(q.y >> 16) * sc)
                                         : make_float4(__uint_as_float(q.x << 16),
                                                       __uint_as_float(q.x & 0xffff0000u),
                                                       __uint_as_float(q.y << 16),
                                                       __uint_as_float(q.y & 0xffff0000u));
                        }
                    }
                }
                }  // S16
                __syncthreads();
                // One trace for all candidates of the thread.  FULL: every
                // window lies inside the trace (trace_span's conservative
                // bounds), so the range test, the zero-pad redirect, the
                // clamp and the per-candidate count are skipped.
                struct Win {
                    int bo[R];    // shared-memory index of each window's first sample
                    float fr[R];  // interpolation fraction
                };
                auto windowsOf = [&](const TraceMeta2 &md, int j, auto fullTag, Win &wn) {
                    constexpr bool FULL = decltype(fullTag)::value;
#pragma unroll
                    for (int qq = 0; qq < NP; qq++) {
                        // traveltime of both candidates of the pair, the
                        // roundings of cmp_time / zocrs_t2 lane by lane
                        const float2 cq = f2(cc[2 * qq], cc[2 * qq + 1]);
                        const float2 hsq2 = f2(md.hsq, md.hsq);
                        float2 t2;
                        float2 t;
                        if constexpr (TT64) {
                            // FP64 squared time; t2 carries only its sign
                            bool pa = zocrs_time_tt64(t0, cc[2 * qq], c1[2 * qq], c2[2 * qq],
                                                      md.dm, md.hsq, &t.x);
                            bool pb = zocrs_time_tt64(t0, cc[2 * qq + 1], c1[2 * qq + 1],
                                                      c2[2 * qq + 1], md.dm, md.hsq, &t.y);
                            t2 = f2(pa ? 1.f : -1.f, pb ? 1.f : -1.f);
                        } else {
                            if (MODEL == kModelCmp) {
                                t2 = __ffma2_rn(cq, hsq2, t0sq2);
                            } else {
                                const float2 dm2 = f2(md.dm, md.dm);
                                const float2 x =
                                    __ffma2_rn(f2(c1[2 * qq], c1[2 * qq + 1]), dm2, t0p2);
                                const float2 bd = __fmul2_rn(f2(c2[2 * qq], c2[2 * qq + 1]), dm2);
                                t2 = __ffma2_rn(cq, hsq2, __ffma2_rn(bd, dm2, __fmul2_rn(x, x)));
                            }
                            if (MODEL == kModelCmp || FULL) {
                                t = f2(sqrtf(t2.x), sqrtf(t2.y));
                            } else {
                                t = f2(sqrtf(fmaxf(t2.x, 0.f)), sqrtf(fmaxf(t2.y, 0.f)));
                            }
                        }
                        // t / dt: the fast-math quotient equals t * (1/dt)
                        // bit for bit, so the reciprocal is taken once
                        const float2 ti = __fmul2_rn(t, rdt2);
                        // k = (int)ti and frac = ti - k without conversions:
                        // for 0 <= ti < 2^23, ti + 2^23 rounded toward zero is
                        // 2^23 + floor(ti) exactly; its bits carry k, and
                        // subtracting 2^23 (exact) gives k as a float
                        const float2 rk = __fadd2_rz(ti, kMagic2);
                        const float2 kf = __fadd2_rn(rk, kNegMagic2);
                        const float2 fq = __ffma2_rn(kf, kNeg1, ti);  // ti - k, exact
#pragma unroll
                        for (int h = 0; h < 2; h++) {
                            const int r = 2 * qq + h;
                            // k - tau (ti >= 2^23, inf: far out of range)
                            const int km = __float_as_int(h ? rk.y : rk.x) - magicTau;
                            wn.fr[r] = h ? fq.y : fq.x;
                            if (FULL) {
                                wn.bo[r] = md.base + km;
                            } else {
                                // k - tau >= 0 && k + tau + 1 < S as one unsigned compare
                                bool in = (unsigned)km < winSpan;
                                if (MODEL != kModelCmp) in = in && (h ? t2.y : t2.x) >= 0;
                                const int b = in ? md.base + km : 0;
#ifdef HPSS_CHECKED
                                if (in && (b < md.base + sm.lo[j] ||
                                           b > md.base + sm.lo[j] + (md.len & kLenMask) - (W + 1)))
                                    atomicOr(a.errorWord, kErrSmemBounds);
#endif
                                // out-of-trace windows read the zero pad: u = 0
                                // for any finite fraction, so the fraction
                                // needs no select
                                wn.bo[r] = (int)min((unsigned)b, (unsigned)kLastBase);
                                used[r] += in ? 1u : 0u;
                            }
                        }
                    }
                };
                // The W + 1 amplitudes of both windows of every pair are loaded
                // into registers before the taps: the loads of one trace issue
                // back to back and the taps run without shared-memory waits.
                auto tapsOf = [&](const Win &wn) {
                    float2 yv[NP][W + 1];
#pragma unroll
                    for (int qq = 0; qq < NP; qq++) {
                        const float *ya = sm.y + wn.bo[2 * qq];
                        const float *yb = sm.y + wn.bo[2 * qq + 1];
#pragma unroll
                        for (int jj = 0; jj <= W; jj++) yv[qq][jj] = f2(ya[jj], yb[jj]);
                    }
#pragma unroll
                    for (int qq = 0; qq < NP; qq++) {
                        const float2 fq = f2(wn.fr[2 * qq], wn.fr[2 * qq + 1]);
#pragma unroll
                        for (int jj = 0; jj < W; jj++) {
                            const float2 y0 = yv[qq][jj];
                            const float2 d = __ffma2_rn(y0, kNeg1, yv[qq][jj + 1]);  // y1 - y0
                            const float2 u = __ffma2_rn(d, fq, y0);  // (y1-y0)*f + y0
                            num[qq][jj] = __fadd2_rn(num[qq][jj], u);
                            if (EXACT_STACK) lin[qq] = __fadd2_rn(lin[qq], u);
                            den[qq] = __ffma2_rn(u, u, den[qq]);
                        }
                    }
                };
#ifdef HPSS_CHECKED
                // the span bounds must hold for every candidate of a FULL trace:
                // recompute its window positions with the scalar arithmetic
                auto checkFull = [&](const TraceMeta2 &md, int j) {
                    if (md.len >= 0) return;
                    for (int r = 0; r < R; r++) {
                        float t2, tt;
                        if (MODEL == kModelCmp) {
                            t2 = __fmaf_rn(cc[r], md.hsq, __fmul_rn(t0, t0));
                            tt = sqrtf(t2);
                        } else if (TT64) {
                            t2 = zocrs_time_tt64(t0, cc[r], c1[r], c2[r], md.dm, md.hsq, &tt)
                                     ? 1.f : -1.f;
                        } else {
                            t2 = zocrs_t2(t0, cc[r], c1[r], c2[r], md.dm, md.hsq);
                            tt = sqrtf(fmaxf(t2, 0.f));
                        }
                        const float ti = __fmul_rn(tt, rdt);
                        const int k = (int)ti;
                        const int b = md.base + k - tau;
                        if ((MODEL != kModelCmp && !(t2 > 0.f)) ||
                            (unsigned)(k - tau) >= winSpan || b < md.base + sm.lo[j] ||
                            b > md.base + sm.lo[j] + (md.len & kLenMask) - (W + 1))
                            atomicOr(a.errorWord, kErrSmemBounds);
                    }
                };
#endif
                // Traces in order.  Two consecutive FULL traces (the common
                // case) are handled together: both traces' window positions
                // first, then the taps of the first and of the second, which
                // gives the scheduler two independent traveltime chains.
                for (int j = 0; j < nkeep;) {
                    const TraceMeta2 mA = sm.meta[j];
                    if (j + 1 < nkeep) {
                        const TraceMeta2 mB = sm.meta[j + 1];
                        if ((mA.len & mB.len) < 0) {
#ifdef HPSS_CHECKED
                            checkFull(mA, j);
                            checkFull(mB, j + 1);
#endif
                            Win wA, wB;
                            windowsOf(mA, j, std::true_type{}, wA);
                            windowsOf(mB, j + 1, std::true_type{}, wB);
                            tapsOf(wA);
                            tapsOf(wB);
                            usedFull += 2;
                            j += 2;
                            continue;
                        }
                    }
#ifdef HPSS_CHECKED
                    checkFull(mA, j);
#endif
                    Win wn;
                    if (mA.len < 0) {
                        windowsOf(mA, j, std::true_type{}, wn);
                        usedFull++;
                    } else {
                        windowsOf(mA, j, std::false_type{}, wn);
                    }
                    tapsOf(wn);
                    j++;
                }
                q0 += nfit;
                if constexpr (COMP) {
                    // fold this round's sums into the compensated totals
                    if (comp) {
#pragma unroll
                        for (int qq = 0; qq < NP; qq++) {
#pragma unroll
                            for (int jj = 0; jj < W; jj++) {
                                two_sum_acc(numT[qq][jj].x, numC[qq][jj].x, num[qq][jj].x);
                                two_sum_acc(numT[qq][jj].y, numC[qq][jj].y, num[qq][jj].y);
                                num[qq][jj] = f2(0.f, 0.f);
                            }
                            two_sum_acc(denT[qq].x, denC[qq].x, den[qq].x);
                            two_sum_acc(denT[qq].y, denC[qq].y, den[qq].y);
                            den[qq] = f2(0.f, 0.f);
                            if (EXACT_STACK) {
                                two_sum_acc(linT[qq].x, linC[qq].x, lin[qq].x);
                                two_sum_acc(linT[qq].y, linC[qq].y, lin[qq].y);
                                lin[qq] = f2(0.f, 0.f);
                            }
                        }
                    }
                }
            }
            if constexpr (COMP) {
                if (comp) {
#pragma unroll
                    for (int qq = 0; qq < NP; qq++) {
#pragma unroll
                        for (int jj = 0; jj < W; jj++)
                            num[qq][jj] = __fadd2_rn(numT[qq][jj], numC[qq][jj]);
                        den[qq] = __fadd2_rn(denT[qq], denC[qq]);
                        lin[qq] = __fadd2_rn(linT[qq], linC[qq]);
                    }
                }
            }

#pragma unroll
            for (int qq = 0; qq < NP; qq++) {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int r = 2 * qq + h;
                    float nm[W];
#pragma unroll
                    for (int jj = 0; jj < W; jj++) nm[jj] = h ? num[qq][jj].y : num[qq][jj].x;
                    float ls = h ? lin[qq].y : lin[qq].x;
                    if (!EXACT_STACK) {
                        ls = 0.f;
#pragma unroll
                        for (int jj = 0; jj < W; jj++) ls += nm[jj];
                    }
                    float sembl, stack;
                    reduce_semblance(nm, ls, h ? den[qq].y : den[qq].x, W, used[r] + usedFull, &sembl,
                                     &stack);
                    const uint32_t p = chunk * a.chunkSize + warp * R + r;
                    if (valid[r]) top2_offer(sembl, best, second);
                    if (valid[r] && sembl > best) {
                        best = sembl;
                        bestStack = stack;
                        bestP = p;
                    }
                }
            }
        }

        sm.bestS[warp][lane] = best;
        sm.bestK[warp][lane] = bestStack;
        sm.bestP[warp][lane] = bestP;
        sm.bestSec[warp][lane] = second;
        __syncthreads();
        if (warp == 0) {
            for (int wv = 1; wv < kTunedWarps; wv++) {
                float os = sm.bestS[wv][lane];
                uint32_t op = sm.bestP[wv][lane];
                if (better(os, op, best, bestP)) bestStack = sm.bestK[wv][lane];
                top2_merge(os, op, sm.bestSec[wv][lane], best, bestP, second);
            }
            if (a.parts > 1) {
                // the merge combines the parts, writes the block and counts ties
                if (s < S) {
                    PartBest pb;
                    pb.best = best;
                    pb.second = second;
                    pb.stack = bestStack;
                    pb.p = bestP;
                    a.partial[((size_t)mi * a.parts + part) * a.S + s] = pb;
                }
            } else {
                if (a.nearTies) {
                    const unsigned tie = __ballot_sync(0xffffffffu, s < S && near_tie(best, second));
                    if (lane == 0 && tie) atomicAdd(a.nearTies, (unsigned long long)__popc(tie));
                }
                if (s < S) {
                    out[s] = best;
                    out[a.S + s] = bestStack;
                    if (bestP != 0xffffffffu) {
                        const float *pr = a.params + (size_t)bestP * np;
                        out[2 * a.S + s] = 2 / sqrtf(pr[0]);
                        for (int j = 1; j < np; j++) out[(size_t)(2 + j) * a.S + s] = pr[j];
                    } else {
                        for (int j = 0; j < np; j++) out[(size_t)(2 + j) * a.S + s] = 0.f;
                    }
                }
            }
        }
        __syncthreads();
    }
}

template <int MODEL, int NP, int MINB, bool EXACT_STACK, int PREC = 0, bool S16 = false>
cudaError_t launch_ls_tuned2_model(const LsParams &p, uint32_t grid,
                                   uint32_t tiles, uint32_t nUnits,
                                   cudaStream_t st) {
    const size_t smem = sizeof(Tuned2Smem<MINB>);
#define HPSS_TUNED2_CASE(WV)                                                  \
    case WV: {                                                                \
        auto k = ls_tuned2_kernel<MODEL, WV, NP, MINB, EXACT_STACK, PREC, S16>; \
        cudaError_t e = cudaFuncSetAttribute(                                 \
            k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);       \
        if (e != cudaSuccess) return e;                                       \
        k<<<grid, kTunedThreads, smem, st>>>(p, tiles, nUnits);              \
        return cudaGetLastError();                                            \
    }
    switch (p.w) {
        HPSS_TUNED2_CASE(1)
        HPSS_TUNED2_CASE(3)
        HPSS_TUNED2_CASE(5)
        HPSS_TUNED2_CASE(7)
        HPSS_TUNED2_CASE(9)
        HPSS_TUNED2_CASE(11)
        HPSS_TUNED2_CASE(13)
        HPSS_TUNED2_CASE(15)
        default:
            return cudaErrorNotSupported;
    }
#undef HPSS_TUNED2_CASE
}

}  // namespace hpss
