// de.cu -- differential evolution per (midpoint, t0 sample), fused.
//
// The reference runs DE/rand/1/bin per sample with one kernel launch and one
// cudaDeviceSynchronize per operator per generation per midpoint
// (DifferentialEvolutionAlgorithm.cpp:21-81, kernels in
// cuda/src/semblance/kernel/common/differential_evolution.cu and the
// {cmp,zocrs,oct}/differential_evolution.cu evaluators).  Here the whole run
// -- initialisation, and per generation mutation, crossover, semblance
// evaluation and selection -- is ONE launch: one thread per individual
// (consecutive threads are the individuals of one sample, the reference's
// thread layout), a CTA holds the whole populations of consecutive samples in
// shared memory, mutation reads the donors from there, and nothing
// round-trips through global memory between operators.
//
// Operator semantics follow the reference:
//  * init: x_j = min_j + U * (max_j - min_j), U in (0, 1]   (startPopulations)
//  * mutation: per parameter j three indices r = trunc(U * (pop - 1)) (not
//    necessarily distinct, may equal i), v_j = x[r1]_j + F (x[r2]_j - x[r3]_j),
//    clamped with fminf(max) then fmaxf(min)                (mutatePopulations)
//  * crossover: l = trunc(U * (nParams - 1)); u_j = (U > CR && l != j) ? x_j
//    : v_j                                                   (crossoverPopulations)
//  * selection: replace when fu.semblance > fx.semblance (strict) (nextGeneration)
//  * `generations` counts the initial evaluation (loop gen = 1 .. G-1)
//  * result: strict '>' scan over individuals from -1 (lowest index wins
//    ties), raw parameters (velocity, not 4/v^2)        (selectBestIndividualsFor*)
// The random stream differs: Philox-4x32-10 (Salmon et al., SC'11), keyed by
// the seed and countered by (midpoint, sample, individual, draw), instead of
// curand XORWOW seeded from time(NULL).  The midpoint enters as its FP32 bit
// pattern, so a midpoint draws the same numbers whatever else its call holds
// (other midpoints, other half-offsets, another process's shard).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "hpss_device.cuh"
#include "hpss_internal.h"
#include "stage.cuh"

namespace hpss {

// ---- Philox-4x32-10 (counter-based RNG; published constants) -------------
struct U4 {
    uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ void mulhilo(uint32_t a, uint32_t b, uint32_t &hi,
                                                 uint32_t &lo) {
    uint64_t p = (uint64_t)a * b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

__host__ __device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo(M0, c.x, hi0, lo0);
        mulhilo(M1, c.z, hi1, lo1);
        U4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// uniform in (0, 1] with 24-bit resolution (curand_uniform's range)
__host__ __device__ __forceinline__ float u01(uint32_t v) {
    return (float)((v >> 8) + 1u) * (1.0f / 16777216.0f);
}

// Stream of uniforms for one individual in one generation.
struct Draws {
    U4 ctr;
    uint32_t k0, k1;
    U4 buf;
    int left;
    __device__ __forceinline__ Draws(uint32_t k0_, uint32_t k1_, uint32_t m0i, uint32_t s,
                                     uint32_t ind, uint32_t gen)
        : k0(k0_), k1(k1_), left(0) {
        ctr.x = gen << 8;
        ctr.y = ind;
        ctr.z = s;
        ctr.w = m0i;
    }
    __device__ __forceinline__ float next() {
        if (left == 0) {
            buf = philox4x32_10(ctr, k0, k1);
            ctr.x++;
            left = 4;
        }
        uint32_t v = left == 4 ? buf.x : left == 3 ? buf.y : left == 2 ? buf.z : buf.w;
        left--;
        return u01(v);
    }
};

__device__ __forceinline__ float2 de_f2(float a, float b) { return make_float2(a, b); }

// OCT: displaced-midpoint tests run side by side per thread, five CTAs per
// SM (before the warp box test, four side by side: OCT DE 2 midpoints 876 ->
// 783 ms; with it, three beat four and two: 3-h0 FP16 DE, 20 generations,
// 2 midpoints 450.2 -> 429.2 ms, two 438.7 ms; four or three CTAs per SM
// 465.8 / 510.7 ms)
constexpr int kDeOctBatch = 3;

// threads of a DE CTA (kDeThreads below), for the per-warp box slots
constexpr int kDeThreadsMax = 256;

// Semblance of one candidate (raw parameters) over the selected traces.
// OCT with boxMode: called by all 32 lanes of the warp (the warp's
// displaced-midpoint box and the tests over blocks of 32 traces are
// collectives); lanes with ev false take part in those only.
template <int MODEL, int W>
__device__ __forceinline__ void de_eval(const DeParams &d, const OctLine &ol, float t0,
                                        float m0, uint32_t first, uint32_t cnt, const float *x,
                                        float *sembl, float *stack, unsigned *notUsed,
                                        bool ev = true, bool boxMode = false) {
    const LsParams &a = d.ls;
    const float v = x[0];
    const float c = 4.0f / (v * v);
    const float p1 = MODEL != kModelCmp ? x[1] : 0.f;
    const float p2 = MODEL == kModelZocrs ? x[2] : 0.f;
    float num[W > 0 ? W : kMaxWindow];
    const int w = W > 0 ? W : a.w;
#pragma unroll
    for (int j = 0; j < (W > 0 ? W : kMaxWindow); j++) num[j] = 0.f;
    float lin = 0.f, den = 0.f;
    unsigned used = 0, nu = 0;
    uint32_t q = 0;
    if (MODEL != kModelOct && W > 0 && !a.selIdx) {
        // CMP / ZO-CRS: two traces per step -- both traveltimes and both
        // windows' loads are issued before the sums, which then take the
        // traces in order (the same sums as one trace at a time)
        // the two traces' traveltimes, floors and window terms in packed
        // f32x2 ops (per lane the same IEEE operations as cmp_time /
        // zocrs_t2 and window_index: t/dt is t*(1/dt) in the fast-math
        // build, and floor(t/dt) is read from the bits of t/dt + 2^23 added
        // toward zero, which (int) gives for 0 <= t/dt < 2^23)
        const float2 c2 = de_f2(c, c), a2 = de_f2(p1, p1), b2 = de_f2(p2, p2);
        const float t0sq = __fmul_rn(t0, t0);
        const float2 t02 = de_f2(t0, t0), t0sq2 = de_f2(t0sq, t0sq);
        const float2 negM02 = de_f2(-m0, -m0);
        const float rdt = 1.0f / a.dt;
        const float2 rdt2 = de_f2(rdt, rdt);
        const float2 kNeg1 = de_f2(-1.f, -1.f);
        const float2 kMagic2 = de_f2(8388608.f, 8388608.f), kNegMagic2 = de_f2(-8388608.f, -8388608.f);
        for (; q + 1 < cnt; q += 2) {
            const uint32_t ti0 = first + q, ti1 = ti0 + 1;
            const float2 hsq2 = de_f2(a.hsq[ti0], a.hsq[ti1]);
            float2 tt2;
            if (MODEL == kModelCmp) {
                tt2 = __ffma2_rn(c2, hsq2, t0sq2);
            } else {
                const float2 dm2 = __fadd2_rn(de_f2(a.mid[ti0], a.mid[ti1]), negM02);  // m - m0
                const float2 x2 = __ffma2_rn(a2, dm2, t02);
                const float2 bd2 = __fmul2_rn(b2, dm2);
                tt2 = __ffma2_rn(c2, hsq2, __ffma2_rn(bd2, dm2, __fmul2_rn(x2, x2)));
            }
            // ZO-CRS: a negative squared time skips the window
            const bool oka = MODEL == kModelCmp || tt2.x >= 0.f;
            const bool okb = MODEL == kModelCmp || tt2.y >= 0.f;
            const float2 t2 = MODEL == kModelCmp
                                  ? de_f2(sqrtf(tt2.x), sqrtf(tt2.y))
                                  : de_f2(sqrtf(fmaxf(tt2.x, 0.f)), sqrtf(fmaxf(tt2.y, 0.f)));
            const float2 ti2 = __fmul2_rn(t2, rdt2);
            const float2 rk = __fadd2_rz(ti2, kMagic2);
            const float2 fq = __ffma2_rn(__fadd2_rn(rk, kNegMagic2), kNeg1, ti2);  // frac
            const int ka = __float_as_int(rk.x) - 0x4B000000;
            const int kb = __float_as_int(rk.y) - 0x4B000000;
            const bool ina = oka && window_in_trace(ka, a.tau, (int)a.S);
            const bool inb = okb && window_in_trace(kb, a.tau, (int)a.S);
            float ya[W > 0 ? W + 1 : 1], yb[W > 0 ? W + 1 : 1];
            if (a.samples16) {
                // 16-bit storage: out-of-trace windows read sample 0 and are
                // zeroed, as the FP32 form's
                load_window(a, ti0, ina ? ka - a.tau : 0, ya);
                load_window(a, ti1, inb ? kb - a.tau : 0, yb);
#pragma unroll
                for (int j = 0; j <= W; j++) {
                    ya[j] = ina ? ya[j] : 0.f;
                    yb[j] = inb ? yb[j] : 0.f;
                }
            } else {
                const float *tra = a.samples + (size_t)ti0 * a.stride + (ina ? ka - a.tau : 0);
                const float *trb = a.samples + (size_t)ti1 * a.stride + (inb ? kb - a.tau : 0);
#pragma unroll
                for (int j = 0; j <= W; j++) {
                    ya[j] = ina ? __ldg(tra + j) : 0.f;
                    yb[j] = inb ? __ldg(trb + j) : 0.f;
                }
            }
            // window terms of both traces: (y1 - y0) * frac + y0 per lane
            float2 u2[W > 0 ? W : 1];
#pragma unroll
            for (int j = 0; j < W; j++) {
                const float2 y0 = de_f2(ya[j], yb[j]);
                const float2 d2 = __ffma2_rn(y0, kNeg1, de_f2(ya[j + 1], yb[j + 1]));
                u2[j] = __ffma2_rn(d2, fq, y0);
            }
            // the sums take trace ti0, then trace ti1; a window outside its
            // trace read zeros (u = 0: it adds nothing) and is not counted;
            // the linear sum is taken from the per-tap sums at the end
#pragma unroll
            for (int j = 0; j < W; j++) {
                const float u = u2[j].x;
                num[j] += u;
                den += u * u;
            }
#pragma unroll
            for (int j = 0; j < W; j++) {
                const float u = u2[j].y;
                num[j] += u;
                den += u * u;
            }
            used += (ina ? 1u : 0u) + (inb ? 1u : 0u);
        }
    }
    // OCT: (t0, candidate) factors once, trace factors from the line's table
    const OctCand kc = oct_cand(t0, c, p1, MODEL == kModelOct ? ol.h0 : 0.f);
    if constexpr (MODEL == kModelOct && W > 0) {
      __shared__ float deBox[kDeThreadsMax / 32][4];  // each warp's displaced-midpoint box
      volatile float *boxSlot = deBox[threadIdx.x >> 5];
      bool boxOn = false;
      if (boxMode) {
          const OctWarpBox box = oct_warp_box(a.octBox, ev, t0, p1, kc, ol.h0);
          boxOn = box.on;
          if (boxOn) oct_box_store(boxSlot, box);
      }
      if (boxOn) {
        // blocks of 32 traces: lane j tests trace qb + j against the warp's
        // displaced-midpoint box, then the lanes evaluate the traces kept, in order
        const int lane = threadIdx.x & 31;
        for (uint32_t qb = 0; qb < cnt; qb += 32) {
            const uint32_t n = min(32u, cnt - qb);
            bool keep = false;
            if ((uint32_t)lane < n) {
                const uint32_t ti = a.selIdx ? a.selIdx[first + qb + lane] : first + qb + lane;
                keep = oct_box_keep(a, ol, ti, boxSlot, m0);
            }
            uint32_t mask = __ballot_sync(0xffffffffu, keep);
            if (ev) nu += n - (uint32_t)__popc(mask);
            while (mask) {
                uint32_t tb[kDeOctBatch];
                bool live[kDeOctBatch];
                const uint32_t firstBit = (uint32_t)__ffs(mask) - 1;
#pragma unroll
                for (int b = 0; b < kDeOctBatch; b++) {
                    live[b] = mask != 0;
                    const uint32_t bit = live[b] ? (uint32_t)__ffs(mask) - 1 : firstBit;
                    if (live[b]) mask &= mask - 1;
                    tb[b] = a.selIdx ? a.selIdx[first + qb + bit] : first + qb + bit;
                }
                if (ev)
                    oct_eval_batch<W, kDeOctBatch>(a, ol, tb, live, kc, c, p1, t0, m0, num,
                                                               lin, den, used, nu);
            }
        }
        q = cnt;
      } else if (!ev) {
        q = cnt;  // a lane without an evaluation only joins the warp's box
      } else {
        // the displaced-midpoint tests of kDeOctBatch traces side by side
        // (independent chains), then the passing traces in order
        for (; q + kDeOctBatch <= cnt; q += kDeOctBatch) {
            uint32_t tb[kDeOctBatch];
            bool live[kDeOctBatch];
#pragma unroll
            for (int b = 0; b < kDeOctBatch; b++) {
                tb[b] = a.selIdx ? a.selIdx[first + q + b] : first + q + b;
                live[b] = true;
            }
            oct_eval_batch<W, kDeOctBatch>(a, ol, tb, live, kc, c, p1, t0, m0, num, lin,
                                                       den, used, nu);
        }
      }
    }
    for (; q < cnt; q++) {
        const uint32_t ti = a.selIdx ? a.selIdx[first + q] : first + q;
        float t;
        int ok;
        if (MODEL == kModelOct) {
            const float4 tf = __ldg(ol.tab + ti);  // {m, gamma^2, 16h^2h0^2, h^2-h0^2}
            ok = oct_model_time(kc, tf.y, tf.z, tf.w, t0, c, p1, tf.x, a.hoff[ti], m0, a.apm,
                                ol.h0, &t);
        } else {
            ok = model_time<MODEL>(t0, c, p1, p2, a.mid[ti], a.hoff[ti], a.hsq[ti], m0, a.apm,
                                   a.h0, &t);
        }
        if (ok < 0) {
            nu++;
            continue;
        }
        if (ok == 0) continue;
        WinIdx wi = window_index(t, a.dt);
        if (window_in_trace(wi.k, a.tau, (int)a.S)) {
            const int k0 = wi.k - a.tau;
            float y1 = amp_at(a, ti, k0);
#pragma unroll
            for (int j = 0; j < (W > 0 ? W : kMaxWindow); j++) {
                if (W == 0 && j >= w) break;
                float y0 = y1;
                y1 = amp_at(a, ti, k0 + j + 1);
                float u = (y1 - y0) * wi.frac + y0;
                num[j] += u;
                lin += u;
                den += u * u;
            }
            used++;
        }
    }
    if (MODEL != kModelOct && W > 0) {
        // CMP / ZO-CRS: the linear sum is the sum of the per-tap sums (the
        // same values added in another order)
        lin = 0.f;
#pragma unroll
        for (int j = 0; j < (W > 0 ? W : 1); j++) lin += num[j];
    }
    reduce_semblance(num, lin, den, w, used, sembl, stack);
    *notUsed += nu;
}

// ---- DE/rand/1/bin operators of one individual ---------------------------
// Initial individual: x_j = min_j + U (max_j - min_j) as one fused
// multiply-add, as the reference's startPopulations compiles.
template <int NP>
__device__ __forceinline__ void de_init_individual(const DeParams &d, uint32_t mkey, uint32_t s,
                                                   uint32_t ind, float (&x)[NP]) {
    Draws rng(d.seedLo, d.seedHi, mkey, s, ind, 0);
#pragma unroll
    for (int j = 0; j < NP; j++) x[j] = __fmaf_rn(rng.next(), __fsub_rn(d.hi[j], d.lo[j]), d.lo[j]);
}

// Trial vector of individual `ind` in generation `gen`: mutation from three
// donors of the sample's population xs (trunc(U (pop - 1)), not necessarily
// distinct), clamped with fminf(max) then fmaxf(min); binomial crossover
// with the parameter l = trunc(U (nParams - 1)) always from the mutant.
template <int NP>
__device__ __forceinline__ void de_trial_vector(const DeParams &d, uint32_t mkey, uint32_t s,
                                                uint32_t ind, uint32_t gen, const float *xs,
                                                const float (&x)[NP], float (&u)[NP]) {
    const uint32_t pop = d.pop;
    Draws rng(d.seedLo, d.seedHi, mkey, s, ind, gen);
    float v[NP];
#pragma unroll
    for (int j = 0; j < NP; j++) {
        const float q1 = rng.next(), q2 = rng.next(), q3 = rng.next();
        const uint32_t r1 = (uint32_t)(q1 * (float)(pop - 1));
        const uint32_t r2 = (uint32_t)(q2 * (float)(pop - 1));
        const uint32_t r3 = (uint32_t)(q3 * (float)(pop - 1));
        float nv = __fmaf_rn(d.F, __fsub_rn(xs[r2 * NP + j], xs[r3 * NP + j]), xs[r1 * NP + j]);
        nv = fminf(nv, d.hi[j]);
        nv = fmaxf(nv, d.lo[j]);
        v[j] = nv;
    }
    const uint32_t l = (uint32_t)(rng.next() * (float)(NP - 1));
#pragma unroll
    for (int j = 0; j < NP; j++) {
        const float r = rng.next();
        u[j] = (r > d.CR && l != (uint32_t)j) ? x[j] : v[j];
    }
}

// ---- CMP / ZO-CRS: the CTA's trials over spans staged in shared memory --
//
// The individuals of a sample sit at scattered parameters, so the windows a
// warp reads from one trace are scattered, and a warp's load from L1 touches
// many cache lines.  Instead the CTA stages, round by round, the sample spans
// of consecutive selected traces that any window of its current trials can
// touch (trace_span over the trials' parameter box and the CTA's t0 range;
// the box is taken anew for every evaluation, so the spans shrink as the
// populations converge) into shared memory -- bulk copies for FP32 rows,
// widening loads for 16-bit rows -- and every thread reads its windows from
// there, and each trace's h^2 and m - m0 from the round's slot (one shared
// word per trace instead of two global loads per thread and trace).  Each
// trial's sums take the same values in the same trace order as de_eval's,
// so the results are the same bit for bit.
constexpr int kDeStageFloats = 9728;   // 38 KB of spans per CTA
constexpr int kDeZeroPad = 16;         // zeros first: windows outside their trace read these

struct DeStage {
    float y[kDeStageFloats];
    float2 hm[kDeThreadsMax];  // per round slot: the trace's h^2 and m - m0 (as m + (-m0))
    int base[kDeThreadsMax];   // per round slot: stage index of the trace's sample 0
    int lo[kDeThreadsMax];
    int len[kDeThreadsMax];
    int full[kDeThreadsMax];  // every window of the trials lies inside the trace
    int warpSum[kDeThreadsMax / 32];
    int warpLen[kDeThreadsMax / 32];
    float boxW[kDeThreadsMax / 32][6];
    unsigned long long bar;  // mbarrier of a round's bulk copies
};

// Stage index of a window's first sample, kept inside the stage (the spans
// hold every window of the trials, so the clamp changes nothing; checked
// builds report a window outside its span).
__device__ __forceinline__ int de_stage_index(int b, int w) {
    return (int)min((unsigned)b, (unsigned)(kDeStageFloats - w - 1));
}

// The CTA-wide (min, max) of every parameter over the trials of its active
// threads: bx holds a thread's own (min, max) pairs of (c, p1, p2) (+inf /
// -inf where it has no trial).  Called by every thread of the CTA.
__device__ __forceinline__ void de_cta_box(DeStage &st, float (&bx)[6], float (&cb)[6]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nWarps = (int)(blockDim.x >> 5);
#pragma unroll
    for (int o = 16; o; o >>= 1) {
#pragma unroll
        for (int j = 0; j < 6; j += 2) {
            bx[j] = fminf(bx[j], __shfl_xor_sync(0xffffffffu, bx[j], o));
            bx[j + 1] = fmaxf(bx[j + 1], __shfl_xor_sync(0xffffffffu, bx[j + 1], o));
        }
    }
    __syncthreads();  // the previous evaluation's last round is read
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < 6; j++) st.boxW[warp][j] = bx[j];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 6; j++) {
        float r = st.boxW[0][j];
        for (int wv = 1; wv < nWarps; wv++)
            r = (j & 1) ? fmaxf(r, st.boxW[wv][j]) : fminf(r, st.boxW[wv][j]);
        cb[j] = r;
    }
}

// One staging round, called by every thread of the CTA: the spans of the
// selected traces q0, q0 + 1, ... (one per thread) that any window of the
// box cb and the t0 range [t0a, t0b] can touch are packed into the stage in
// trace order, as many as fit, and copied (bulk copies for FP32 rows,
// widening loads for 16-bit rows); slot j of the stage holds trace q0 + j.
// Returns the traces staged; 0 when a span is longer than the stage (the
// host stages only rows that fit; reported in the error word), -1 when the
// copies did not complete in time (reported; every thread gets -1).
template <int MODEL>
__device__ int de_stage_round(const DeParams &d, DeStage &st, uint32_t &phase,
                              const float (&cb)[6], bool anyActive, float t0a, float t0b,
                              float m0, uint32_t first, uint32_t cnt, uint32_t q0) {
    const LsParams &a = d.ls;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nWarps = (int)(blockDim.x >> 5);
        // spans of the next traces, one per thread, packed in trace order
        const uint32_t q = q0 + threadIdx.x;
        int lo = 0, len = 0;
        bool full = false;
        float tm = 0.f, thsq = 0.f;
        if (q < cnt) {
            tm = a.mid[first + q];
            thsq = a.hsq[first + q];
            if (anyActive) trace_span<MODEL>(a, cb, m0, t0a, t0b, tm, thsq, &lo, &len, &full);
        }
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int vv = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += vv;
        }
        if (lane == 31) st.warpSum[warp] = incl;
        __syncthreads();  // also: the previous round's windows are read
        int off = kDeZeroPad + incl - len;
        for (int wv = 0; wv < warp; wv++) off += st.warpSum[wv];
        // the spans that fit form a prefix of the threads (offsets only grow)
        const bool fits = q < cnt && off + len <= kDeStageFloats;
        const int keptLen = __reduce_add_sync(0xffffffffu, fits ? len : 0);
        if (lane == 0) st.warpLen[warp] = keptLen;
        if (fits) {
            st.base[threadIdx.x] = off - lo;
            st.lo[threadIdx.x] = lo;
            st.len[threadIdx.x] = len;
            st.full[threadIdx.x] = full ? 1 : 0;
            // the evaluation's per-trace inputs, read from here instead of
            // from global memory by every thread (m - m0 rounded as there)
            st.hm[threadIdx.x] = make_float2(thsq, __fadd_rn(tm, -m0));
        }
        const uint32_t nfit = (uint32_t)__syncthreads_count(fits);
        if (nfit == 0) {
            // a span longer than the stage (the host stages only rows that fit)
            if (threadIdx.x == 0) atomicOr(a.errorWord, kErrSpanOverflow);
            return 0;
        }
        if (a.samples16 == nullptr) {
            if (threadIdx.x == 0) {
                uint32_t floats = 0;
                for (int wv = 0; wv < nWarps; wv++) floats += (uint32_t)st.warpLen[wv];
                stage_bar_expect(&st.bar, floats * 4u);
            }
            if (fits && len > 0) {
                // the previous round's reads are ordered before the async-proxy writes
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                stage_bulk_copy(st.y + off, a.samples + (size_t)(first + q) * a.stride + lo,
                                (uint32_t)len * 4u, &st.bar);
            }
            const bool ok = stage_bar_wait(&st.bar, phase, 1u << 22);
            phase ^= 1u;
            if (__syncthreads_or(!ok)) {
                // report, wait (again bounded) for this CTA's copies in flight
                if (threadIdx.x == 0) atomicOr(a.errorWord, kErrTimeout);
                stage_bar_wait(&st.bar, phase ^ 1u, 1u << 22);
                return -1;
            }
        } else {
            // 16-bit rows: a warp per trace, 4 samples per 8-byte load, widened
            // to FP32 as load_window widens them
            for (uint32_t j = (uint32_t)warp; j < nfit; j += (uint32_t)nWarps) {
                const int lj = st.lo[j], nj = st.len[j];
                const uint32_t ti = first + q0 + j;
                float4 *dst = reinterpret_cast<float4 *>(st.y + st.base[j] + lj);
                const uint2 *src =
                    reinterpret_cast<const uint2 *>(a.samples16 + (size_t)ti * a.stride + lj);
                const float sc = a.storage == 2 ? __ldg(a.scale + ti) : 1.f;
                for (int vv = lane; vv < (nj >> 2); vv += 32) {
                    const uint2 w4 = __ldg(src + vv);
                    dst[vv] = a.storage == 2
                                  ? make_float4(half_bits_to_float(w4.x & 0xffffu) * sc,
                                                half_bits_to_float(w4.x >> 16) * sc,
                                                half_bits_to_float(w4.y & 0xffffu) * sc,
                                                half_bits_to_float(w4.y >> 16) * sc)
                                  : make_float4(__uint_as_float(w4.x << 16),
                                                __uint_as_float(w4.x & 0xffff0000u),
                                                __uint_as_float(w4.y << 16),
                                                __uint_as_float(w4.y & 0xffff0000u));
                }
            }
            __syncthreads();
        }
    return (int)nfit;
}

// Called by every thread of the CTA (inactive threads stage and synchronise
// only).  False when a round's copies did not complete in time (reported in
// the error word); every thread then gets false.
template <int MODEL, int W>
__device__ bool de_eval_staged(const DeParams &d, DeStage &st, uint32_t &phase, float t0,
                               float t0a, float t0b, float m0, uint32_t first, uint32_t cnt,
                               bool active, const float *x, float *sembl, float *stack) {
    const LsParams &a = d.ls;
    const float v = x[0];
    const float c = 4.0f / (v * v);
    const float p1 = MODEL != kModelCmp ? x[1] : 0.f;
    const float p2 = MODEL == kModelZocrs ? x[2] : 0.f;
    // the active trials' parameter box: (c, p1, p2), min and max
    const float inf = __int_as_float(0x7f800000);
    float bx[6] = {active ? c : inf,  active ? c : -inf,  active ? p1 : inf,
                   active ? p1 : -inf, active ? p2 : inf, active ? p2 : -inf};
    float cb[6];
    de_cta_box(st, bx, cb);
    const bool anyActive = cb[0] <= cb[1];

    float num[W];
#pragma unroll
    for (int j = 0; j < W; j++) num[j] = 0.f;
    float den = 0.f;
    unsigned used = 0;
    const float2 c2 = de_f2(c, c), a2 = de_f2(p1, p1), b2 = de_f2(p2, p2);
    const float t0sq = __fmul_rn(t0, t0);
    const float2 t02 = de_f2(t0, t0), t0sq2 = de_f2(t0sq, t0sq);
    const float rdt = 1.0f / a.dt;
    // windows whose start k - tau keeps the whole window inside the trace
    const unsigned winSpan = (int)a.S > 2 * a.tau + 1 ? (unsigned)((int)a.S - 2 * a.tau - 1) : 0u;
    const float2 rdt2 = de_f2(rdt, rdt);
    const float2 kNeg1 = de_f2(-1.f, -1.f);
    const float2 kMagic2 = de_f2(8388608.f, 8388608.f), kNegMagic2 = de_f2(-8388608.f, -8388608.f);
    for (uint32_t q0 = 0; q0 < cnt;) {
        const int staged = de_stage_round<MODEL>(d, st, phase, cb, anyActive, t0a, t0b, m0,
                                                  first, cnt, q0);
        if (staged < 0) return false;
        if (staged == 0) break;
        const uint32_t nfit = (uint32_t)staged;
        if (active) {
            // two traces per step, as de_eval: both traveltimes and floors in
            // packed f32x2 ops, both windows read before the sums, which take
            // the traces in order.  FULL: every window of the CTA's trials
            // lies inside both traces (trace_span's conservative bounds, for
            // ZO-CRS with every squared time positive), so the range tests,
            // the zero-pad redirect and the per-trace count are skipped (the
            // same sums: those tests pass for every window)
            auto pairStep = [&](uint32_t j, auto fullTag) {
                constexpr bool FULL = decltype(fullTag)::value;
                const float2 hmA = st.hm[j], hmB = st.hm[j + 1];
                const float2 hsq2 = de_f2(hmA.x, hmB.x);
                float2 tt2;
                if (MODEL == kModelCmp) {
                    tt2 = __ffma2_rn(c2, hsq2, t0sq2);
                } else {
                    const float2 dm2 = de_f2(hmA.y, hmB.y);  // m + (-m0), both traces
                    const float2 x2 = __ffma2_rn(a2, dm2, t02);
                    const float2 bd2 = __fmul2_rn(b2, dm2);
                    tt2 = __ffma2_rn(c2, hsq2, __ffma2_rn(bd2, dm2, __fmul2_rn(x2, x2)));
                }
                const bool oka = MODEL == kModelCmp || tt2.x >= 0.f;
                const bool okb = MODEL == kModelCmp || tt2.y >= 0.f;
                const float2 t2 = (MODEL == kModelCmp || FULL)
                                      ? de_f2(sqrtf(tt2.x), sqrtf(tt2.y))
                                      : de_f2(sqrtf(fmaxf(tt2.x, 0.f)), sqrtf(fmaxf(tt2.y, 0.f)));
                const float2 ti2 = __fmul2_rn(t2, rdt2);
                const float2 rk = __fadd2_rz(ti2, kMagic2);
                const float2 fq = __ffma2_rn(__fadd2_rn(rk, kNegMagic2), kNeg1, ti2);  // frac
                const int ka = __float_as_int(rk.x) - 0x4B000000;
                const int kb = __float_as_int(rk.y) - 0x4B000000;
                // k - tau >= 0 && k + tau + 1 < S as one unsigned compare
                const bool ina = FULL || (oka && (unsigned)(ka - a.tau) < winSpan);
                const bool inb = FULL || (okb && (unsigned)(kb - a.tau) < winSpan);
#ifdef HPSS_CHECKED
                if ((ina && (ka - a.tau < st.lo[j] || ka - a.tau + W >= st.lo[j] + st.len[j])) ||
                    (inb && (kb - a.tau < st.lo[j + 1] ||
                             kb - a.tau + W >= st.lo[j + 1] + st.len[j + 1])))
                    atomicOr(a.errorWord, kErrSmemBounds);
                if (FULL && !(oka && okb && window_in_trace(ka, a.tau, (int)a.S) &&
                              window_in_trace(kb, a.tau, (int)a.S)))
                    atomicOr(a.errorWord, kErrSmemBounds);
#endif
                // a window outside its trace reads the zero pad (u = 0); the
                // clamp keeps every read inside the stage whatever the span
                const float *ya = st.y + de_stage_index(ina ? st.base[j] + ka - a.tau : 0, W);
                const float *yb = st.y + de_stage_index(inb ? st.base[j + 1] + kb - a.tau : 0, W);
                float2 u2[W];
                float y0a = ya[0], y0b = yb[0];
#pragma unroll
                for (int jj = 0; jj < W; jj++) {
                    const float y1a = ya[jj + 1], y1b = yb[jj + 1];
                    const float2 y0 = de_f2(y0a, y0b);
                    const float2 dd = __ffma2_rn(y0, kNeg1, de_f2(y1a, y1b));
                    u2[jj] = __ffma2_rn(dd, fq, y0);
                    y0a = y1a;
                    y0b = y1b;
                }
#pragma unroll
                for (int jj = 0; jj < W; jj++) {
                    num[jj] += u2[jj].x;
                    den += u2[jj].x * u2[jj].x;
                }
#pragma unroll
                for (int jj = 0; jj < W; jj++) {
                    num[jj] += u2[jj].y;
                    den += u2[jj].y * u2[jj].y;
                }
                used += FULL ? 2u : (ina ? 1u : 0u) + (inb ? 1u : 0u);
            };
            uint32_t j = 0;
            for (; j + 1 < nfit; j += 2) {
                // the same for every thread of the CTA: no divergence
                if (st.full[j] & st.full[j + 1])
                    pairStep(j, std::true_type{});
                else
                    pairStep(j, std::false_type{});
            }
            if (j < nfit) {
                // an odd trace at the end of the round: de_eval's one-trace step
                const uint32_t ti = first + q0 + j;
                float t;
                const int ok = model_time<MODEL>(t0, c, p1, p2, a.mid[ti], a.hoff[ti], a.hsq[ti],
                                                 m0, a.apm, a.h0, &t);
                if (ok > 0) {
                    const WinIdx wi = window_index(t, a.dt);
                    if (window_in_trace(wi.k, a.tau, (int)a.S)) {
#ifdef HPSS_CHECKED
                        if (wi.k - a.tau < st.lo[j] || wi.k - a.tau + W >= st.lo[j] + st.len[j])
                            atomicOr(a.errorWord, kErrSmemBounds);
#endif
                        const float *yr = st.y + de_stage_index(st.base[j] + wi.k - a.tau, W);
                        float y1 = yr[0];
#pragma unroll
                        for (int jj = 0; jj < W; jj++) {
                            const float y0 = y1;
                            y1 = yr[jj + 1];
                            const float u = (y1 - y0) * wi.frac + y0;
                            num[jj] += u;
                            den += u * u;
                        }
                        used++;
                    }
                }
            }
        }
        q0 += nfit;
    }
    // the linear sum is the sum of the per-tap sums, as in de_eval
    float lin = 0.f;
#pragma unroll
    for (int j = 0; j < W; j++) lin += num[j];
    reduce_semblance(num, lin, den, W, used, sembl, stack);
    return true;
}

// Two trials per thread (individuals 2i and 2i + 1 of a sample) over the
// staged spans: per trace, both trials' traveltimes, floors, window terms
// and sums run in packed f32x2 ops, each half carrying one trial with the
// same IEEE operations, in the same trace order, as de_eval_staged gives it
// alone -- the same sums bit for bit, with one instruction for both trials
// where de_eval_staged issues one per trial for the sums.  Called by every
// thread of the CTA; act[k] false: no trial k (staging and synchronisation
// only).  False when a round's copies did not complete in time.
template <int MODEL, int W>
__device__ bool de_eval_staged2(const DeParams &d, DeStage &st, uint32_t &phase, float t0,
                                float t0a, float t0b, float m0, uint32_t first, uint32_t cnt,
                                const bool (&act)[2], const float (&x0)[MODEL == kModelCmp ? 1 : 3],
                                const float (&x1)[MODEL == kModelCmp ? 1 : 3], float (&sembl)[2],
                                float (&stack)[2]) {
    const LsParams &a = d.ls;
    const float cA = 4.0f / (x0[0] * x0[0]), cB = 4.0f / (x1[0] * x1[0]);
    const float pA = MODEL != kModelCmp ? x0[MODEL != kModelCmp ? 1 : 0] : 0.f;
    const float pB = MODEL != kModelCmp ? x1[MODEL != kModelCmp ? 1 : 0] : 0.f;
    const float qA = MODEL == kModelZocrs ? x0[MODEL == kModelZocrs ? 2 : 0] : 0.f;
    const float qB = MODEL == kModelZocrs ? x1[MODEL == kModelZocrs ? 2 : 0] : 0.f;
    const float inf = __int_as_float(0x7f800000);
    auto lo2 = [&](float u, float v) { return fminf(act[0] ? u : inf, act[1] ? v : inf); };
    auto hi2 = [&](float u, float v) { return fmaxf(act[0] ? u : -inf, act[1] ? v : -inf); };
    float bx[6] = {lo2(cA, cB), hi2(cA, cB), lo2(pA, pB), hi2(pA, pB), lo2(qA, qB), hi2(qA, qB)};
    float cb[6];
    de_cta_box(st, bx, cb);
    const bool anyActive = cb[0] <= cb[1];

    float2 num[W];
#pragma unroll
    for (int j = 0; j < W; j++) num[j] = de_f2(0.f, 0.f);
    float2 den = de_f2(0.f, 0.f);
    unsigned usedA = 0, usedB = 0;
    const float2 c2 = de_f2(cA, cB), a2 = de_f2(pA, pB), b2 = de_f2(qA, qB);
    const float t0sq = __fmul_rn(t0, t0);
    const float2 t02 = de_f2(t0, t0), t0sq2 = de_f2(t0sq, t0sq);
    const float rdt = 1.0f / a.dt;
    // windows whose start k - tau keeps the whole window inside the trace
    const unsigned winSpan = (int)a.S > 2 * a.tau + 1 ? (unsigned)((int)a.S - 2 * a.tau - 1) : 0u;
    const float2 rdt2 = de_f2(rdt, rdt);
    const float2 kNeg1 = de_f2(-1.f, -1.f);
    const float2 kMagic2 = de_f2(8388608.f, 8388608.f), kNegMagic2 = de_f2(-8388608.f, -8388608.f);
    const bool anyOwn = act[0] || act[1];
    for (uint32_t q0 = 0; q0 < cnt;) {
        const int staged = de_stage_round<MODEL>(d, st, phase, cb, anyActive, t0a, t0b, m0,
                                                  first, cnt, q0);
        if (staged < 0) return false;
        if (staged == 0) break;
        const uint32_t nfit = (uint32_t)staged;
        if (anyOwn) {
            // FULL: every window of the CTA's trials lies inside the trace
            // (the range tests, zero-pad redirect and count are skipped)
            auto traceStep = [&](uint32_t j, auto fullTag) {
                constexpr bool FULL = decltype(fullTag)::value;
                const float2 hm = st.hm[j];  // h^2, m + (-m0): de_eval_staged's rounding
                const float2 hsq2 = de_f2(hm.x, hm.x);
                float2 tt2;
                if (MODEL == kModelCmp) {
                    tt2 = __ffma2_rn(c2, hsq2, t0sq2);
                } else {
                    const float2 dm2 = de_f2(hm.y, hm.y);
                    const float2 xx = __ffma2_rn(a2, dm2, t02);
                    const float2 bd2 = __fmul2_rn(b2, dm2);
                    tt2 = __ffma2_rn(c2, hsq2, __ffma2_rn(bd2, dm2, __fmul2_rn(xx, xx)));
                }
                const bool oka = MODEL == kModelCmp || tt2.x >= 0.f;
                const bool okb = MODEL == kModelCmp || tt2.y >= 0.f;
                const float2 t2 = (MODEL == kModelCmp || FULL)
                                      ? de_f2(sqrtf(tt2.x), sqrtf(tt2.y))
                                      : de_f2(sqrtf(fmaxf(tt2.x, 0.f)), sqrtf(fmaxf(tt2.y, 0.f)));
                const float2 ti2 = __fmul2_rn(t2, rdt2);
                const float2 rk = __fadd2_rz(ti2, kMagic2);
                const float2 fq = __ffma2_rn(__fadd2_rn(rk, kNegMagic2), kNeg1, ti2);  // frac
                const int ka = __float_as_int(rk.x) - 0x4B000000;
                const int kb = __float_as_int(rk.y) - 0x4B000000;
                // k - tau >= 0 && k + tau + 1 < S as one unsigned compare
                const bool ina = FULL || (oka && (unsigned)(ka - a.tau) < winSpan);
                const bool inb = FULL || (okb && (unsigned)(kb - a.tau) < winSpan);
                const int base = st.base[j];
#ifdef HPSS_CHECKED
                if ((act[0] && ina && (ka - a.tau < st.lo[j] || ka - a.tau + W >= st.lo[j] + st.len[j])) ||
                    (act[1] && inb && (kb - a.tau < st.lo[j] || kb - a.tau + W >= st.lo[j] + st.len[j])))
                    atomicOr(a.errorWord, kErrSmemBounds);
                if (FULL && ((act[0] && !(oka && window_in_trace(ka, a.tau, (int)a.S))) ||
                             (act[1] && !(okb && window_in_trace(kb, a.tau, (int)a.S)))))
                    atomicOr(a.errorWord, kErrSmemBounds);
#endif
                // a window outside its trace reads the zero pad (u = 0); the
                // clamp keeps every read inside the stage whatever the span
                const float *ya = st.y + de_stage_index(ina ? base + ka - a.tau : 0, W);
                const float *yb = st.y + de_stage_index(inb ? base + kb - a.tau : 0, W);
                float y0a = ya[0], y0b = yb[0];
#pragma unroll
                for (int jj = 0; jj < W; jj++) {
                    const float y1a = ya[jj + 1], y1b = yb[jj + 1];
                    const float2 y0 = de_f2(y0a, y0b);
                    const float2 dd = __ffma2_rn(y0, kNeg1, de_f2(y1a, y1b));
                    const float2 u = __ffma2_rn(dd, fq, y0);
                    num[jj] = __fadd2_rn(num[jj], u);
                    den = __ffma2_rn(u, u, den);
                    y0a = y1a;
                    y0b = y1b;
                }
                usedA += FULL || ina ? 1u : 0u;
                usedB += FULL || inb ? 1u : 0u;
            };
            for (uint32_t j = 0; j < nfit; j++) {
                if (st.full[j])  // the same for every thread of the CTA
                    traceStep(j, std::true_type{});
                else
                    traceStep(j, std::false_type{});
            }
        }
        q0 += nfit;
    }
    // per trial: the linear sum is the sum of the per-tap sums, as in de_eval
#pragma unroll
    for (int k = 0; k < 2; k++) {
        float nm[W];
        float lin = 0.f;
#pragma unroll
        for (int j = 0; j < W; j++) {
            nm[j] = k ? num[j].y : num[j].x;
            lin += nm[j];
        }
        reduce_semblance(nm, lin, k ? den.y : den.x, W, k ? usedB : usedA, &sembl[k], &stack[k]);
    }
    return true;
}

// CMP / ZO-CRS with staged spans and an even population: two individuals
// per thread (2i and 2i + 1 of one sample; a CTA holds `spc` whole
// populations of consecutive samples, 2 x threads individuals), evaluated
// together by de_eval_staged2.  Every individual draws its own counter-based
// stream and runs the same operators as in de_kernel, so the results are
// de_kernel's bit for bit.
template <int MODEL, int W>
__global__ void __launch_bounds__(kDeThreadsMax, 4)
de_pair_kernel(DeParams d, uint32_t spc, uint32_t groups, uint32_t nUnits) {
    constexpr int NP = MODEL == kModelCmp ? 1 : 3;
    const LsParams &a = d.ls;
    extern __shared__ __align__(16) float deSmem[];
    const uint32_t pop = d.pop, half = pop / 2;
    float *X = deSmem;                           // [spc][pop][NP]
    float *FX = deSmem + (size_t)spc * pop * NP; // [spc][pop] (final argmax)
    float *FK = FX + (size_t)spc * pop;          // [spc][pop]
    DeStage *stg = reinterpret_cast<DeStage *>(
        deSmem + (((size_t)spc * pop * (NP + 2) + 3) & ~(size_t)3));
    uint32_t stagePhase = 0;
    if (threadIdx.x < kDeZeroPad) stg->y[threadIdx.x] = 0.f;
    if (threadIdx.x == 0) stage_bar_init(&stg->bar);
    __syncthreads();
    const uint32_t ls = threadIdx.x / half;      // sample within the CTA
    const uint32_t pi = threadIdx.x % half;      // individuals 2 pi, 2 pi + 1
    const bool member = ls < spc;                // threads past spc * half only sync
    const uint32_t ind[2] = {2 * pi, 2 * pi + 1};
    __shared__ uint32_t nextUnit;
    for (uint32_t unit = blockIdx.x;; unit += gridDim.x) {
        if (a.unitCounter) {
            __syncthreads();  // every thread has read the previous unit
            if (threadIdx.x == 0) nextUnit = atomicAdd(a.unitCounter, 1u);
            __syncthreads();
            unit = nextUnit;
        }
        if (unit >= nUnits) break;
        const uint32_t mi = a.order ? a.order[unit / groups] : unit / groups;
        const uint32_t s = (unit % groups) * spc + ls;
        const bool active = member && s < a.S;
        const bool act[2] = {active, active};
        const float m0 = a.m0s[mi];
        const uint32_t first = a.selFirst[mi], cnt = a.selCount[mi];
        const uint32_t mkey = __float_as_uint(m0);
        const float t0 = static_cast<float>(active ? s : 0) * a.dt;
        const float t0a = static_cast<float>((unit % groups) * spc) * a.dt;
        const float t0b = static_cast<float>(min((unit % groups) * spc + spc - 1, a.S - 1)) * a.dt;
        float *xs = X + (size_t)(member ? ls : 0) * pop * NP;  // this sample's population
        // the population (xs) and its fitness and stack (FX, FK) live in
        // shared memory; a thread holds only its two trial vectors
        float *fx = FX + (size_t)(member ? ls : 0) * pop;
        float *fk = FK + (size_t)(member ? ls : 0) * pop;
        // ---- initial population and its fitness (generation 1)
        {
            float x[2][NP];
#pragma unroll
            for (int k = 0; k < 2; k++) {
                if (active) {
                    de_init_individual<NP>(d, mkey, s, ind[k], x[k]);
#pragma unroll
                    for (int j = 0; j < NP; j++) xs[ind[k] * NP + j] = x[k][j];
                } else {
#pragma unroll
                    for (int j = 0; j < NP; j++) x[k][j] = d.lo[j];
                }
            }
            float f[2], fs[2];
            if (!de_eval_staged2<MODEL, W>(d, *stg, stagePhase, t0, t0a, t0b, m0, first, cnt, act,
                                           x[0], x[1], f, fs))
                return;  // copies timed out (error word); every thread leaves
            if (member) {
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    fx[ind[k]] = active ? f[k] : -1.f;
                    fk[ind[k]] = active ? fs[k] : 0.f;
                }
            }
        }
        // ---- generations 2 .. G
        for (uint32_t gen = 1; gen < d.gens; gen++) {
            __syncthreads();  // population of the previous generation complete
            float u[2][NP];
#pragma unroll
            for (int k = 0; k < 2; k++) {
                float x[NP];
#pragma unroll
                for (int j = 0; j < NP; j++) x[j] = active ? xs[ind[k] * NP + j] : d.lo[j];
#pragma unroll
                for (int j = 0; j < NP; j++) u[k][j] = x[j];
                if (active) de_trial_vector<NP>(d, mkey, s, ind[k], gen, xs, x, u[k]);
            }
            __syncthreads();  // every donor read before any replacement
            float fu[2], fuk[2];
            if (!de_eval_staged2<MODEL, W>(d, *stg, stagePhase, t0, t0a, t0b, m0, first, cnt, act,
                                           u[0], u[1], fu, fuk))
                return;
            if (active) {
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    if (fu[k] > fx[ind[k]]) {
#pragma unroll
                        for (int j = 0; j < NP; j++) xs[ind[k] * NP + j] = u[k][j];
                        fx[ind[k]] = fu[k];
                        fk[ind[k]] = fuk[k];
                    }
                }
            }
        }
        // ---- best individual per sample: strict '>' from -1 in index order
        __syncthreads();
        if (active && pi == 0) {
            float best = -1.f, bestK = 0.f;
            uint32_t bi = 0xffffffffu;
            for (uint32_t i = 0; i < pop; i++) {
                const float f = FX[ls * pop + i];
                if (f > best) {
                    best = f;
                    bestK = FK[ls * pop + i];
                    bi = i;
                }
            }
            float *out = a.out + (size_t)mi * (2 + NP) * a.S;
            out[s] = best;
            out[a.S + s] = bestK;
#pragma unroll
            for (int j = 0; j < NP; j++)
                out[(size_t)(2 + j) * a.S + s] = bi != 0xffffffffu ? xs[bi * NP + j] : 0.f;
        }
        __syncthreads();  // shared memory reused by the next unit
    }
}

// One thread per individual.  A CTA holds `spc` whole populations of
// consecutive samples of one midpoint (thread = sample-in-CTA * pop +
// individual, the reference's thread layout), so every lane works for any
// population size; the population vectors live in shared memory, where
// mutation reads the three donors.  Persistent over (midpoint, sample
// group) units, taken from a work queue (heaviest midpoints first) when a
// call has more units than resident CTAs.
constexpr int kDeThreads = kDeThreadsMax;

// OCT: five resident CTAs per SM (48 registers) -- its evaluation waits on
// long dependent square-root / reciprocal chains, so resident warps and the
// batched displaced-midpoint tests (kDeOctBatch) both pay.  CMP / ZO-CRS: four (64 registers), which
// their two-trace steps fit without spills (ZO-CRS DE, 2 midpoints: 41.9 ->
// 38.1 ms; 16 midpoints unchanged; three- or four-trace steps and a 6-CTA
// bound are slower).
template <int MODEL, int W>
__global__ void __launch_bounds__(kDeThreads, MODEL == kModelOct ? 5 : 4)
de_kernel(DeParams d, uint32_t spc, uint32_t groups, uint32_t nUnits) {
    constexpr int NP = MODEL == kModelCmp ? 1 : (MODEL == kModelZocrs ? 3 : 2);
    const LsParams &a = d.ls;
    extern __shared__ __align__(16) float deSmem[];
    const uint32_t pop = d.pop;
    float *X = deSmem;                           // [spc][pop][NP]
    float *FX = deSmem + (size_t)spc * pop * NP; // [spc][pop] (final argmax)
    float *FK = FX + (size_t)spc * pop;          // [spc][pop]
    // OCT: evaluations assigned by slope rank (de_sorted_smem_floats)
    float *TR = FK + (size_t)spc * pop;                 // [threads][NP] trial vectors
    float *KEY = TR + (size_t)blockDim.x * NP;          // [threads] sort key
    float *RES = KEY + blockDim.x;                      // [threads][2] fitness, stack
    uint32_t *PERM = reinterpret_cast<uint32_t *>(RES + 2 * (size_t)blockDim.x);
    __shared__ unsigned long long nuCta;
    // CMP / ZO-CRS with staged spans: the stage follows the populations
    constexpr bool kStaged = MODEL != kModelOct && W > 0;
    const bool staged = kStaged && d.staged;
    DeStage *stg = reinterpret_cast<DeStage *>(
        deSmem + (((size_t)spc * pop * (NP + 2) + 3) & ~(size_t)3));
    uint32_t stagePhase = 0;
    if (staged) {
        if (threadIdx.x < kDeZeroPad) stg->y[threadIdx.x] = 0.f;
        if (threadIdx.x == 0) stage_bar_init(&stg->bar);
        __syncthreads();
    }
    const uint32_t ls = threadIdx.x / pop;       // sample within the CTA
    const uint32_t ind = threadIdx.x % pop;      // individual
    const bool member = ls < spc;                // threads past spc * pop only sync

    // OCT: whether a trace passes the displaced-midpoint test depends on the
    // candidate (mostly on its slope), and a warp runs the OCT time and
    // window path for a trace as soon as one lane passes.  So the CTA's
    // evaluations are dealt by slope rank: thread r evaluates the trial of
    // the member with the r-th smallest slope (any sample of the CTA), and
    // the fitness goes back to its owner through shared memory.  Every
    // trial's fitness is computed exactly as by its owner.  Called by all
    // threads of the CTA.
    auto evalSorted = [&](const float *trial, bool active, float s0f, float m0,
                          const OctLine &ol, uint32_t first, uint32_t cnt, float *f, float *fk,
                          unsigned *notUsed) {
#pragma unroll
        for (int j = 0; j < NP; j++) TR[threadIdx.x * NP + j] = trial[j];
        const float key = active ? trial[NP - 1] : __int_as_float(0x7f800000);  // slope; +inf
        KEY[threadIdx.x] = key;
        __syncthreads();
        uint32_t rank = 0;
        for (uint32_t t = 0; t < blockDim.x; t++) {
            const float kt = KEY[t];
            rank += (kt < key || (kt == key && t < threadIdx.x)) ? 1u : 0u;
        }
        PERM[rank] = threadIdx.x;
        __syncthreads();
        const uint32_t o = PERM[threadIdx.x];  // the member whose trial this thread evaluates
        const bool ev = KEY[o] != __int_as_float(0x7f800000);
        const float t0o = (s0f + static_cast<float>(o / pop)) * a.dt;
        // OCT: all lanes enter when the box test is on (warp collectives)
        const bool boxMode = MODEL == kModelOct && W > 0 && a.octBox;
        if (boxMode || ev) {
            float fo, fko;
            de_eval<MODEL, W>(d, ol, t0o, m0, first, cnt, TR + o * NP, &fo, &fko, notUsed, ev,
                              boxMode);
            if (ev) {
                RES[2 * o] = fo;
                RES[2 * o + 1] = fko;
            }
        }
        __syncthreads();
        *f = RES[2 * threadIdx.x];
        *fk = RES[2 * threadIdx.x + 1];
    };

    __shared__ uint32_t nextUnit;
    for (uint32_t unit = blockIdx.x;; unit += gridDim.x) {
        // work queue (heaviest midpoints first when ordered), else round-robin
        if (a.unitCounter) {
            __syncthreads();  // every thread has read the previous unit
            if (threadIdx.x == 0) nextUnit = atomicAdd(a.unitCounter, 1u);
            __syncthreads();
            unit = nextUnit;
        }
        if (unit >= nUnits) break;
        const uint32_t mi = a.order ? a.order[unit / groups] : unit / groups;
        const uint32_t s = (unit % groups) * spc + ls;
        const bool active = member && s < a.S;
        const float m0 = a.m0s[mi];
        const uint32_t first = a.selFirst[mi], cnt = a.selCount[mi];
        const OctLine ol = oct_line(a, mi);          // OCT: the midpoint's h0 and table
        const uint32_t mkey = __float_as_uint(m0);   // random-stream key of the midpoint
        const float t0 = static_cast<float>(active ? s : 0) * a.dt;
        const float s0f = static_cast<float>((unit % groups) * spc);  // the CTA's first sample
        // the t0 range of the CTA's samples (staged spans)
        const float t0a = s0f * a.dt;
        const float t0b = static_cast<float>(min((unit % groups) * spc + spc - 1, a.S - 1)) * a.dt;
        float *xs = X + (size_t)(member ? ls : 0) * pop * NP;  // this sample's population
        float x[NP];
        float fx = -1.f, fxk = 0.f;
        unsigned notUsed = 0;
        if (threadIdx.x == 0) nuCta = 0;
        // ---- initial population and its fitness (generation 1)
        if (active) {
            de_init_individual<NP>(d, mkey, s, ind, x);
#pragma unroll
            for (int j = 0; j < NP; j++) xs[ind * NP + j] = x[j];
            if (MODEL != kModelOct && !staged)
                de_eval<MODEL, W>(d, ol, t0, m0, first, cnt, x, &fx, &fxk, &notUsed);
        } else {
#pragma unroll
            for (int j = 0; j < NP; j++) x[j] = d.lo[j];
        }
        if constexpr (kStaged) {
            if (staged) {
                float f0, k0;
                if (!de_eval_staged<MODEL, W>(d, *stg, stagePhase, t0, t0a, t0b, m0, first, cnt,
                                              active, x, &f0, &k0))
                    return;  // copies timed out (error word); every thread leaves
                if (active) {
                    fx = f0;
                    fxk = k0;
                }
            }
        }
        if (MODEL == kModelOct) {
            evalSorted(x, active, s0f, m0, ol, first, cnt, &fx, &fxk, &notUsed);
            if (!active) fx = -1.f;
        }
        // ---- generations 2 .. G
        for (uint32_t gen = 1; gen < d.gens; gen++) {
            __syncthreads();  // population of the previous generation complete
            float u[NP];
#pragma unroll
            for (int j = 0; j < NP; j++) u[j] = x[j];
            if (active) de_trial_vector<NP>(d, mkey, s, ind, gen, xs, x, u);
            __syncthreads();  // every donor read before any replacement
            float fu = -1.f, fuk = 0.f;
            if (MODEL == kModelOct)
                evalSorted(u, active, s0f, m0, ol, first, cnt, &fu, &fuk, &notUsed);
            if constexpr (kStaged) {
                if (staged && !de_eval_staged<MODEL, W>(d, *stg, stagePhase, t0, t0a, t0b, m0,
                                                        first, cnt, active, u, &fu, &fuk))
                    return;  // copies timed out (error word); every thread leaves
            }
            if (active) {
                if (MODEL != kModelOct && !staged)
                    de_eval<MODEL, W>(d, ol, t0, m0, first, cnt, u, &fu, &fuk, &notUsed);
                if (fu > fx) {
#pragma unroll
                    for (int j = 0; j < NP; j++) {
                        x[j] = u[j];
                        xs[ind * NP + j] = u[j];
                    }
                    fx = fu;
                    fxk = fuk;
                }
            }
        }
        // ---- best individual per sample: strict '>' from -1 in index order
        if (member) {
            FX[ls * pop + ind] = fx;
            FK[ls * pop + ind] = fxk;
        }
        __syncthreads();
        if (MODEL == kModelOct && notUsed) atomicAdd(&nuCta, (unsigned long long)notUsed);
        if (active && ind == 0) {
            float best = -1.f, bestK = 0.f;
            uint32_t bi = 0xffffffffu;
            for (uint32_t i = 0; i < pop; i++) {
                const float f = FX[ls * pop + i];
                if (f > best) {
                    best = f;
                    bestK = FK[ls * pop + i];
                    bi = i;
                }
            }
            float *out = a.out + (size_t)mi * (2 + NP) * a.S;
            out[s] = best;
            out[a.S + s] = bestK;
#pragma unroll
            for (int j = 0; j < NP; j++)
                out[(size_t)(2 + j) * a.S + s] = bi != 0xffffffffu ? xs[bi * NP + j] : 0.f;
        }
        __syncthreads();
        if (MODEL == kModelOct && threadIdx.x == 0 && a.notUsed && nuCta)
            atomicAdd(a.notUsed + mi, nuCta);
        __syncthreads();  // shared memory reused by the next unit
    }
}

// OCT trace selection with the initial DE population
// (selectTracesForOffsetContinuationTrajectoryAndDifferentialEvolution,
// oct/differential_evolution.cu:130-168): a trace is used if any (sample,
// initial individual) gives a valid displaced midpoint within apm.  The
// initial individuals are regenerated from the counter-based stream.  One
// warp per (midpoint, candidate trace) slot over the whole GPU writes a 0 / 1
// flag into the slot (d.ls.selFirst: the prefix of candCount); the flags are
// then compacted in order (launch_select_compact).
// Per (midpoint, sample): the slope and c = 4/v^2 ranges of the initial
// population (the box the selection's per-sample box test takes).
__global__ void de_select_boxes_kernel(DeParams d, float4 *boxes) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const LsParams &a = d.ls;
    if (i >= (uint64_t)a.nM0 * a.S) return;
    const uint32_t mi = (uint32_t)(i / a.S), s = (uint32_t)(i % a.S);
    const uint32_t mkey = __float_as_uint(a.m0s[mi]);
    const float inf = __int_as_float(0x7f800000);
    float4 b = make_float4(inf, -inf, inf, -inf);
    for (uint32_t ind = 0; ind < d.pop; ind++) {
        Draws rng(d.seedLo, d.seedHi, mkey, s, ind, 0);
        const float v = __fmaf_rn(rng.next(), __fsub_rn(d.hi[0], d.lo[0]), d.lo[0]);
        const float sl = __fmaf_rn(rng.next(), __fsub_rn(d.hi[1], d.lo[1]), d.lo[1]);
        const float c = 4.0f / (v * v);
        b.x = fminf(b.x, sl);
        b.y = fmaxf(b.y, sl);
        b.z = fminf(b.z, c);
        b.w = fmaxf(b.w, c);
    }
    boxes[i] = b;
}

// Lanes first take 32 samples at a time through the box test of their
// sample's initial population (boxes; oct_sample_may_pass): only samples the
// box cannot rule out go through the per-individual tests, whose results
// are the flags.
__global__ void de_select_oct_flags_kernel(DeParams d, const uint32_t *candFirst,
                                           uint64_t total, uint32_t *selIdx,
                                           const float4 *boxes) {
    const LsParams &a = d.ls;
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
    const OctLine ol = oct_line(a, mi);
    const float h0 = ol.h0;
    const uint32_t mkey = __float_as_uint(m0);
    const float m = a.mid[ti], h = a.hoff[ti];
    const float4 tf = __ldg(ol.tab + ti);
    const float4 *mbox = boxes + (size_t)mi * a.S;
    bool used = false;
    for (uint32_t s0 = 0; s0 < a.S && !used; s0 += 32) {
        const uint32_t sl0 = s0 + lane;
        bool may = false;
        if (sl0 < a.S) {
            const float4 b = mbox[sl0];
            // (HPSS_OCT_BOX_TEST=0: every sample tested)
            may = !a.octBox || oct_sample_may_pass(tf, h, h0, static_cast<float>(sl0) * a.dt,
                                                   b.x, b.y, b.z, b.w, m0, a.apm);
        }
        for (uint32_t mask = __ballot_sync(0xffffffffu, may); mask && !used;
             mask &= mask - 1) {
            const uint32_t s = s0 + __ffs(mask) - 1;
            const float t0 = static_cast<float>(s) * a.dt;
            for (uint32_t i0 = 0; i0 < d.pop && !used; i0 += 32) {
                const uint32_t ind = i0 + lane;
                bool hit = false;
                if (ind < d.pop) {
                    Draws rng(d.seedLo, d.seedHi, mkey, s, ind, 0);
                    const float v = __fmaf_rn(rng.next(), __fsub_rn(d.hi[0], d.lo[0]), d.lo[0]);
                    const float sl =
                        __fmaf_rn(rng.next(), __fsub_rn(d.hi[1], d.lo[1]), d.lo[1]);
                    const float c = 4.0f / (v * v);
                    float mh;
                    const int e = oct_displaced_midpoint(h, h0, t0, m0, c, sl, &mh);
                    hit = (e == DE_OK && fabsf(m - mh) <= a.apm);
                }
                used = __any_sync(0xffffffffu, hit);
            }
        }
    }
    if (lane == 0) selIdx[g] = used ? 1u : 0u;
}

size_t de_smem_bytes(uint32_t spc, uint32_t pop, int np) {
    return (size_t)spc * pop * (np + 2) * sizeof(float);
}

template <int MODEL, int W>
cudaError_t launch_de_w(const DeParams &d, uint32_t numSms, uint32_t spc, uint32_t threads,
                        uint32_t groups, uint64_t units, size_t smem, cudaStream_t st) {
    int perSm = 0;
    cudaError_t e = cudaFuncSetAttribute(de_kernel<MODEL, W>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, de_kernel<MODEL, W>, (int)threads,
                                                      smem);
    if (e != cudaSuccess) return e;
    const uint32_t grid =
        (uint32_t)std::min<uint64_t>(units, (uint64_t)numSms * (uint64_t)std::max(perSm, 1));
    // one wave: every unit has its own CTA, the work queue only adds latency
    DeParams q = d;
    if (units <= grid) q.ls.unitCounter = nullptr;
    de_kernel<MODEL, W><<<grid, threads, smem, st>>>(q, spc, groups, (uint32_t)units);
    return cudaGetLastError();
}

template <int MODEL, int W>
cudaError_t launch_de_pair_w(const DeParams &d, uint32_t numSms, uint32_t spc, uint32_t threads,
                             uint32_t groups, uint64_t units, size_t smem, cudaStream_t st) {
    int perSm = 0;
    cudaError_t e = cudaFuncSetAttribute(de_pair_kernel<MODEL, W>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, de_pair_kernel<MODEL, W>,
                                                      (int)threads, smem);
    if (e != cudaSuccess) return e;
    const uint32_t grid =
        (uint32_t)std::min<uint64_t>(units, (uint64_t)numSms * (uint64_t)std::max(perSm, 1));
    DeParams q = d;
    if (units <= grid) q.ls.unitCounter = nullptr;
    de_pair_kernel<MODEL, W><<<grid, threads, smem, st>>>(q, spc, groups, (uint32_t)units);
    return cudaGetLastError();
}

// CMP / ZO-CRS with staged spans and an even population: two individuals per
// thread (HPSS_DE_PAIRS=0: one, de_kernel; =1: two even for calls too small
// to fill a wave; the same results either way)
template <int MODEL>
cudaError_t launch_de_pairs(const DeParams &d, uint32_t numSms, cudaStream_t st) {
    constexpr int NP = MODEL == kModelCmp ? 1 : 3;
    const uint32_t pop = d.pop;
    const uint32_t spc = std::max<uint32_t>(1u, 2u * kDeThreads / pop);
    const uint32_t threads = ((spc * pop / 2 + 31) / 32) * 32;
    const uint32_t groups = (d.ls.S + spc - 1) / spc;
    const uint64_t units = (uint64_t)d.ls.nM0 * groups;
    if (units == 0) return cudaSuccess;
    if (units > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    const size_t smem = ((de_smem_bytes(spc, pop, NP) + 15) & ~(size_t)15) + sizeof(DeStage);
    switch (d.ls.w) {
        case 1: return launch_de_pair_w<MODEL, 1>(d, numSms, spc, threads, groups, units, smem, st);
        case 3: return launch_de_pair_w<MODEL, 3>(d, numSms, spc, threads, groups, units, smem, st);
        case 5: return launch_de_pair_w<MODEL, 5>(d, numSms, spc, threads, groups, units, smem, st);
        case 7: return launch_de_pair_w<MODEL, 7>(d, numSms, spc, threads, groups, units, smem, st);
        case 9: return launch_de_pair_w<MODEL, 9>(d, numSms, spc, threads, groups, units, smem, st);
        case 11: return launch_de_pair_w<MODEL, 11>(d, numSms, spc, threads, groups, units, smem, st);
        default: return cudaErrorNotSupported;
    }
}

template <int MODEL>
cudaError_t launch_de_model(const DeParams &d, uint32_t numSms, cudaStream_t st) {
    constexpr int NP = MODEL == kModelCmp ? 1 : (MODEL == kModelZocrs ? 3 : 2);
    const uint32_t pop = d.pop;
    uint32_t spc = pop >= (uint32_t)kDeThreads ? 1u : kDeThreads / pop;
    // HPSS_DE_SAMPLES_PER_CTA: fewer samples (whole populations) per CTA
    // (smaller CTAs, each generation barrier over fewer warps)
    if (const char *env = std::getenv("HPSS_DE_SAMPLES_PER_CTA")) {
        const int v = std::atoi(env);
        if (v >= 1 && (uint32_t)v < spc) spc = (uint32_t)v;
    }
    const uint32_t threads = ((spc * pop + 31) / 32) * 32;
    const uint32_t groups = (d.ls.S + spc - 1) / spc;
    const uint64_t units = (uint64_t)d.ls.nM0 * groups;
    if (units == 0) return cudaSuccess;
    if (units > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    // OCT adds the slope-sorted evaluation's regions: trial vectors, keys,
    // fitness / stack pairs and the permutation, one each per thread
    // CMP / ZO-CRS: windows from spans staged in shared memory when a whole
    // row fits the stage (HPSS_DE_STAGED=0: read through L1 instead; the
    // results are the same bit for bit)
    DeParams q = d;
    const char *stagedEnv = std::getenv("HPSS_DE_STAGED");
    q.staged = MODEL != kModelOct && d.ls.w >= 1 && d.ls.w <= 11 && !d.ls.selIdx &&
               d.ls.stride + kDeZeroPad <= (uint32_t)kDeStageFloats &&
               !(stagedEnv && std::strcmp(stagedEnv, "0") == 0);
    size_t smem = de_smem_bytes(spc, pop, NP) +
                  (MODEL == kModelOct ? (size_t)threads * (NP + 4) * sizeof(float) : 0);
    if (q.staged) smem = ((smem + 15) & ~(size_t)15) + sizeof(DeStage);
    if constexpr (MODEL != kModelOct) {
        // two individuals per thread halve the CTAs of a call (twice the
        // samples per CTA): taken when the call still fills a wave of four
        // CTAs per SM, so that small calls keep every SM busy
        const char *pairEnv = std::getenv("HPSS_DE_PAIRS");
        const uint32_t pairSpc = std::max<uint32_t>(1u, 2u * kDeThreads / pop);
        const uint64_t pairUnits = (uint64_t)d.ls.nM0 * ((d.ls.S + pairSpc - 1) / pairSpc);
        const bool forced = pairEnv && std::strcmp(pairEnv, "1") == 0;
        if (q.staged && pop % 2 == 0 && !(pairEnv && std::strcmp(pairEnv, "0") == 0) &&
            (forced || pairUnits >= (uint64_t)numSms * 4))
            return launch_de_pairs<MODEL>(q, numSms, st);
    }
    switch (d.ls.w) {
        case 1: return launch_de_w<MODEL, 1>(q, numSms, spc, threads, groups, units, smem, st);
        case 3: return launch_de_w<MODEL, 3>(q, numSms, spc, threads, groups, units, smem, st);
        case 5: return launch_de_w<MODEL, 5>(q, numSms, spc, threads, groups, units, smem, st);
        case 7: return launch_de_w<MODEL, 7>(q, numSms, spc, threads, groups, units, smem, st);
        case 9: return launch_de_w<MODEL, 9>(q, numSms, spc, threads, groups, units, smem, st);
        case 11: return launch_de_w<MODEL, 11>(q, numSms, spc, threads, groups, units, smem, st);
        default: return launch_de_w<MODEL, 0>(q, numSms, spc, threads, groups, units, smem, st);
    }
}

cudaError_t launch_de(const DeParams &d, int model, uint32_t numSms, cudaStream_t st) {
    if (model == kModelCmp) return launch_de_model<kModelCmp>(d, numSms, st);
    if (model == kModelZocrs) return launch_de_model<kModelZocrs>(d, numSms, st);
    return launch_de_model<kModelOct>(d, numSms, st);
}

cudaError_t launch_de_select_oct(const DeParams &d, const uint32_t *candFirst,
                                 const uint32_t *candCount, uint32_t *selIdx,
                                 uint32_t *selCount, uint64_t total, float4 *boxes,
                                 cudaStream_t st) {
    if (d.ls.nM0 == 0) return cudaSuccess;
    if (total > 0) {
        const uint64_t nb = (uint64_t)d.ls.nM0 * d.ls.S;
        de_select_boxes_kernel<<<(uint32_t)((nb + 255) / 256), 256, 0, st>>>(d, boxes);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        const uint64_t blocks = (total * 32 + 255) / 256;
        if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
        de_select_oct_flags_kernel<<<(uint32_t)blocks, 256, 0, st>>>(d, candFirst, total,
                                                                     selIdx, boxes);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return launch_select_compact(d.ls, candFirst, candCount, selIdx, selCount, st);
}

}  // namespace hpss
