// ls_oct.cu -- the tuned linear-search kernel for the OCT traveltime.
//
// OCT differs from CMP / ZO-CRS in where the time goes: per (sample,
// candidate, trace) the displaced midpoint (oct/common.cuh:7-35) and, for the
// traces that pass |m - mh| <= apm, the OCT time (:37-94) cost a few square
// roots and divisions each, while most traces of the wide OCT aperture fail
// the test and read no samples at all.  Staging trace spans in shared memory
// does not pay here (the spans are whole traces and mostly unused), so this
// kernel reads the windows it needs through L1:
//
//  * lane = t0 sample (32 consecutive samples per warp): neighbouring lanes
//    have nearly the same displaced midpoint and window position, so the skip
//    decisions agree across the warp and the window loads fall on a few
//    cache lines of one trace row;
//  * a thread evaluates one candidate at a time (resident warps, not chains
//    in one thread, hide the latency);
//  * the candidate range is split into `parts` ((midpoint, 32-sample tile,
//    part) units) so that a call with few midpoints still fills the GPU, and
//    every unit into warp units (one per warp slot, see ls_oct_kernel); each
//    warp unit writes the best / runner-up of its candidates and
//    merge_parts_kernel combines them in candidate order;
//  * a call with more units than resident CTAs takes the warp units from a
//    work queue, heaviest midpoints first;
//  * a warp drops, per block of 32 traces, those no sample of its tile can
//    pass (oct_warp_box / oct_box_keep) before the per-sample tests.
//
// The per-candidate arithmetic is the plain kernel's (model_time<kModelOct>,
// window_index, the COMPUTE_SEMBLANCE restatement), in the same trace order,
// so semblance, stack and chosen candidate equal the plain kernel's; the OCT
// formulas take their per-trace factors from the line's factor table and
// their (t0, candidate) factors from registers (the same roundings).
#include "hpss_device.cuh"
#include "hpss_internal.h"

namespace hpss {

constexpr int kOctWarps = 8;

// One candidate per thread: the kernel waits on dependent square-root /
// reciprocal chains, so resident warps pay more than candidates in one
// thread, and the smaller candidate chunks give small calls more units
// (against two candidates per thread, OCT DE line geometry, 11 x 5
// candidates: 4.07 -> 3.10 ms on one midpoint, 12.1 -> 10.0 ms on four).
// The displaced-midpoint tests of kOctMhBatch traces run side by side
// (independent chains) before the passing traces are taken in order, four
// CTAs per SM (before the warp box test, four side by side: 3.10 -> 2.77 ms
// on one midpoint; with it, two beat four and three: 3.24 / 9.60 / 38.7 ms
// -> 3.17 / 9.48 / 38.0 ms on 1 / 4 / 16 midpoints, three 3.27 / 9.73 /
// 39.2 ms).
constexpr int kOctMhBatch = 2;

// Warp units: a (midpoint, 32-sample tile, candidate part) unit is split
// into kOctWarps warp units, warp slot k taking candidates chunk * kOctWarps + k
// of the part's chunks; every warp unit writes its own best / runner-up
// (partial[mi][part][slot][S]) and merge_parts_kernel combines all of them
// in candidate order.  Warps never wait for each other: the candidates keep
// different numbers of traces (their slopes decide the displaced-midpoint
// tests), and a CTA-wide merge per unit would hold every warp until the
// slowest one is done.  Warp units are taken from the work queue one warp
// at a time; without the queue CTA b's warps take the slots of units b,
// b + grid, ... (the warps of a CTA read the same trace rows).
//
// TT64 (precision mode HPSS_PREC_FP64_TRAVELTIME): every trace the box test
// keeps gets the displaced midpoint and time in FP64 (oct_time_f64, the
// plain kernel's form: same bits), one trace at a time; the box test's
// margins cover the FP32 forms, and the FP64 values lie closer to the exact
// ones.
template <int W, bool TT64>
__global__ void __launch_bounds__(kOctWarps * 32, 4)
ls_oct_kernel(LsParams a, uint32_t tiles, uint32_t parts, uint32_t chunksPerPart,
              uint32_t nWarpUnits, PartBest *partial) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int S = (int)a.S, tau = a.tau;
    const uint32_t nChunks = (a.P + kOctWarps - 1) / kOctWarps;
    __shared__ float shBox[kOctWarps][4];  // each warp's displaced-midpoint box
    // each warp's block of 32 traces as its box test read them: table entry,
    // half-offset, trace index (the evaluation takes them from here)
    __shared__ float4 blkTab[kOctWarps][32];
    __shared__ float blkHoff[kOctWarps][32];
    __shared__ uint32_t blkTi[kOctWarps][32];
    for (uint32_t k = 0;; k++) {
        uint32_t wu;
        if (a.unitCounter) {
            uint32_t got = 0;
            if (lane == 0) got = atomicAdd(a.unitCounter, 1u);
            wu = __shfl_sync(0xffffffffu, got, 0);
        } else {
            wu = (blockIdx.x + k * gridDim.x) * kOctWarps + warp;
        }
        if (wu >= nWarpUnits) break;
        const uint32_t slot = wu % kOctWarps, unit = wu / kOctWarps;
        const uint32_t part = unit % parts;
        const uint32_t tile = (unit / parts) % tiles;
        const uint32_t mi = a.order ? a.order[unit / (parts * tiles)] : unit / (parts * tiles);
        const int s = (int)tile * 32 + lane;
        const int sc = min(s, S - 1);
        const float t0 = static_cast<float>(sc) * a.dt;
        const float m0 = a.m0s[mi];
        const uint32_t first = a.selFirst[mi], cnt = a.selCount[mi];
        const OctLine ol = oct_line(a, mi);  // the midpoint's h0 and factor table

        float best = -1.f, second = -1.f, bestStack = 0.f;
        uint32_t bestP = 0xffffffffu;
        unsigned long long notUsed = 0;
        const uint32_t c0 = part * chunksPerPart;
        const uint32_t c1 = min(c0 + chunksPerPart, nChunks);
        for (uint32_t chunk = c0; chunk < c1; chunk++) {
            const uint32_t p = chunk * kOctWarps + slot;
            if (p >= a.P) break;
            const float cc = a.params[2 * (size_t)p];
            const float sl = a.params[2 * (size_t)p + 1];
            const OctCand kc = oct_cand(t0, cc, sl, ol.h0);  // (t0, candidate) factors
            // the warp's displaced-midpoint box (oct_warp_box)
            bool boxOn;
            {
                const OctWarpBox box = oct_warp_box(a.octBox, true, t0, sl, kc, ol.h0);
                boxOn = box.on;
                if (boxOn) oct_box_store(shBox[warp], box);
            }
            float num[W];
#pragma unroll
            for (int j = 0; j < W; j++) num[j] = 0.f;
            float lin = 0.f, den = 0.f;
            unsigned used = 0, nu = 0;
            // FP64 traveltime of one trace (TT64), then its window
            auto evalTt64 = [&](uint32_t ti) {
                float t;
                const int ok = oct_time_f64(t0, cc, sl, a.mid[ti], a.hoff[ti], m0, a.apm, ol.h0, &t);
                if (ok < 0) {
                    nu++;
                    return;
                }
                if (ok == 0) return;
                const WinIdx wi = window_index(t, a.dt);
                if (window_in_trace(wi.k, tau, S)) {
                    accum_window<W>(a, ti, wi.k - tau, wi.frac, num, lin, den);
                    used++;
                }
            };
            if (boxOn) {
                // blocks of 32 traces: lane j tests trace qb + j for the whole
                // warp, then the warp evaluates the traces kept, in order
                for (uint32_t qb = 0; qb < cnt; qb += 32) {
                    const uint32_t n = min(32u, cnt - qb);
                    bool keep = false;
                    if ((uint32_t)lane < n) {
                        const uint32_t ti = a.selIdx ? a.selIdx[first + qb + lane] : first + qb + lane;
                        const float4 tf = __ldg(ol.tab + ti);
                        const float hf = __ldg(a.hoff + ti);
                        keep = oct_box_keep_tf(a, ol, tf, hf, shBox[warp], m0);
                        blkTab[warp][lane] = tf;
                        blkHoff[warp][lane] = hf;
                        blkTi[warp][lane] = ti;
                    }
                    uint32_t mask = __ballot_sync(0xffffffffu, keep);
                    __syncwarp();  // the block's slots written before they are read
                    nu += n - (uint32_t)__popc(mask);
                    if constexpr (TT64) {
                        for (; mask; mask &= mask - 1) {
                            const uint32_t bit = (uint32_t)__ffs(mask) - 1;
                            evalTt64(a.selIdx ? a.selIdx[first + qb + bit] : first + qb + bit);
                        }
                    }
                    while (mask) {
                        OctBlockTraces<kOctMhBatch> tr;
                        tr.tab = blkTab[warp];
                        tr.hoffs = blkHoff[warp];
                        tr.ti = blkTi[warp];
                        bool live[kOctMhBatch];
                        const uint32_t firstBit = (uint32_t)__ffs(mask) - 1;
#pragma unroll
                        for (int bb = 0; bb < kOctMhBatch; bb++) {
                            live[bb] = mask != 0;
                            tr.bit[bb] = live[bb] ? (uint32_t)__ffs(mask) - 1 : firstBit;
                            if (live[bb]) mask &= mask - 1;
                        }
                        oct_eval_traces<W, kOctMhBatch>(a, ol, tr, live, kc, cc, sl, t0, m0, num,
                                                        lin, den, used, nu);
                    }
                    __syncwarp();  // the block's slots read before the next block writes them
                }
            } else {
                // displaced-midpoint tests of kOctMhBatch traces side by side,
                // then the passing traces in order; the rest one by one
                uint32_t q = 0;
                if constexpr (TT64) {
                    for (; q < cnt; q++) evalTt64(a.selIdx ? a.selIdx[first + q] : first + q);
                }
                for (; q + kOctMhBatch <= cnt; q += kOctMhBatch) {
                    uint32_t tb[kOctMhBatch];
                    bool live[kOctMhBatch];
#pragma unroll
                    for (int bb = 0; bb < kOctMhBatch; bb++) {
                        tb[bb] = a.selIdx ? a.selIdx[first + q + bb] : first + q + bb;
                        live[bb] = true;
                    }
                    oct_eval_batch<W, kOctMhBatch>(a, ol, tb, live, kc, cc, sl, t0, m0, num, lin, den,
                                                   used, nu);
                }
                for (; q < cnt; q++) {
                    uint32_t tb[kOctMhBatch];
                    bool live[kOctMhBatch];
#pragma unroll
                    for (int bb = 0; bb < kOctMhBatch; bb++) {
                        tb[bb] = a.selIdx ? a.selIdx[first + q] : first + q;
                        live[bb] = bb == 0;
                    }
                    oct_eval_batch<W, kOctMhBatch>(a, ol, tb, live, kc, cc, sl, t0, m0, num, lin, den,
                                                   used, nu);
                }
            }
            float sembl, stack;
            reduce_semblance(num, lin, den, W, used, &sembl, &stack);
            top2_offer(sembl, best, second);
            if (sembl > best) {
                best = sembl;
                bestStack = stack;
                bestP = p;
            }
            if (s < S) notUsed += nu;
        }
        if (s < S) {
            PartBest pb;
            pb.best = best;
            pb.second = second;
            pb.stack = bestStack;
            pb.p = bestP;
            partial[(((size_t)mi * parts + part) * kOctWarps + slot) * a.S + s] = pb;
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) notUsed += __shfl_xor_sync(0xffffffffu, notUsed, o);
        if (lane == 0 && notUsed && a.notUsed) atomicAdd(a.notUsed + mi, notUsed);
    }
}

// Combine the parts of every (midpoint, sample) in candidate order; write the
// result block and count near-ties (also used by the pair kernel's split).
__global__ void merge_parts_kernel(LsParams a, uint32_t parts, const PartBest *partial) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < (uint64_t)a.nM0 * a.S;
    bool tie = false;
    if (live) {
        const uint32_t mi = (uint32_t)(i / a.S), s = (uint32_t)(i % a.S);
        const int np = a.np;
        float *out = a.out + (size_t)mi * (2 + np) * a.S;
        if (a.selCount[mi] == 0) {
            // reference: midpoint skipped, reset (zero) result
            for (int r = 0; r < 2 + np; r++) out[(size_t)r * a.S + s] = 0.f;
        } else {
            float best = -1.f, second = -1.f, stack = 0.f;
            uint32_t bp = 0xffffffffu;
            for (uint32_t k = 0; k < parts; k++) {
                const PartBest pb = partial[((size_t)mi * parts + k) * a.S + s];
                if (better(pb.best, pb.p, best, bp)) stack = pb.stack;
                top2_merge(pb.best, pb.p, pb.second, best, bp, second);
            }
            out[s] = best;
            out[a.S + s] = stack;
            if (bp != 0xffffffffu) {
                const float *pr = a.params + (size_t)bp * np;
                out[2 * a.S + s] = 2 / sqrtf(pr[0]);
                for (int j = 1; j < np; j++) out[(size_t)(2 + j) * a.S + s] = pr[j];
            } else {
                for (int j = 0; j < np; j++) out[(size_t)(2 + j) * a.S + s] = 0.f;
            }
            tie = near_tie(best, second);
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, tie);
    if ((threadIdx.x & 31) == 0 && m && a.nearTies)
        atomicAdd(a.nearTies, (unsigned long long)__popc(m));
}

cudaError_t launch_merge_parts(const LsParams &p, uint32_t parts, const PartBest *partial,
                               cudaStream_t st) {
    const uint64_t n = (uint64_t)p.nM0 * p.S;
    if (n == 0) return cudaSuccess;
    merge_parts_kernel<<<(uint32_t)((n + 255) / 256), 256, 0, st>>>(p, parts, partial);
    return cudaGetLastError();
}

__global__ void oct_trace_table_kernel(const float *mid, const float *hoff, uint32_t n,
                                       float h0, float4 *tab) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const OctTrace f = oct_trace(hoff[i], h0);
    tab[i] = make_float4(mid[i], f.gs, f.p16h, f.dif);
}

cudaError_t launch_oct_trace_table(const float *mid, const float *hoff, uint32_t n, float h0,
                                   float4 *tab, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    oct_trace_table_kernel<<<(n + 255) / 256, 256, 0, st>>>(mid, hoff, n, h0, tab);
    return cudaGetLastError();
}

size_t oct_partial_bytes(uint32_t nM0, uint32_t S, uint32_t parts) {
    return (size_t)nM0 * parts * kOctWarps * S * sizeof(PartBest);
}

template <int R>
uint32_t oct_chunks(uint32_t P) {
    return (P + kOctWarps * R - 1) / (kOctWarps * R);
}

template <int W, bool TT64>
cudaError_t launch_oct_w(const LsParams &p, uint32_t numSms, void *partial, uint32_t parts,
                         cudaStream_t st) {
    const uint32_t tiles = (p.S + 31) / 32;
    const uint32_t nChunks = oct_chunks<1>(p.P);
    const uint32_t chunksPerPart = (nChunks + parts - 1) / parts;
    const uint64_t units = (uint64_t)p.nM0 * tiles * parts;
    if (units == 0) return cudaSuccess;
    // warp-unit indices (and the queue counter past the last unit) stay below 2^31
    if (units * kOctWarps > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    int perSm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, ls_oct_kernel<W, TT64>,
                                                                  kOctWarps * 32, 0);
    if (e != cudaSuccess) return e;
    const uint32_t grid =
        (uint32_t)std::min<uint64_t>(units, (uint64_t)numSms * (uint64_t)std::max(perSm, 1));
    // one wave: every unit has its own CTA, the work queue only adds latency
    LsParams q = p;
    if (units <= grid) q.unitCounter = nullptr;
    ls_oct_kernel<W, TT64><<<grid, kOctWarps * 32, 0, st>>>(
        q, tiles, parts, chunksPerPart, (uint32_t)(units * kOctWarps),
        static_cast<PartBest *>(partial));
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_merge_parts(p, parts * kOctWarps, static_cast<const PartBest *>(partial), st);
}

// Parts: enough (midpoint, tile, part) units for ~8 waves of the GPU, never
// more than the candidate chunks.
uint32_t oct_parts(const LsParams &p, uint32_t numSms) {
    constexpr int R = 1;
    const uint32_t tiles = (p.S + 31) / 32;
    const uint64_t base = (uint64_t)p.nM0 * tiles;
    const uint64_t want = (uint64_t)numSms * 2 * 8;
    uint64_t parts = base >= want ? 1 : (want + base - 1) / base;
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(parts, oct_chunks<R>(p.P)));
}

template <bool TT64>
cudaError_t launch_ls_oct_t(const LsParams &p, uint32_t numSms, void *partial, uint32_t parts,
                            cudaStream_t st) {
    switch (p.w) {
        case 1: return launch_oct_w<1, TT64>(p, numSms, partial, parts, st);
        case 3: return launch_oct_w<3, TT64>(p, numSms, partial, parts, st);
        case 5: return launch_oct_w<5, TT64>(p, numSms, partial, parts, st);
        case 7: return launch_oct_w<7, TT64>(p, numSms, partial, parts, st);
        case 9: return launch_oct_w<9, TT64>(p, numSms, partial, parts, st);
        case 11: return launch_oct_w<11, TT64>(p, numSms, partial, parts, st);
        case 13: return launch_oct_w<13, TT64>(p, numSms, partial, parts, st);
        case 15: return launch_oct_w<15, TT64>(p, numSms, partial, parts, st);
        default: return cudaErrorNotSupported;
    }
}

cudaError_t launch_ls_oct(const LsParams &p, uint32_t numSms, void *partial, uint32_t parts,
                          cudaStream_t st, bool tt64) {
    return tt64 ? launch_ls_oct_t<true>(p, numSms, partial, parts, st)
                : launch_ls_oct_t<false>(p, numSms, partial, parts, st);
}

}  // namespace hpss
