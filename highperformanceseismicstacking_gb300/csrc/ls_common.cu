// ls_common.cu -- small kernels around the linear search: candidate grid,
// per-chunk candidate bounds, OCT trace selection, storage conversion.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "hpss_device.cuh"
#include "hpss_internal.h"

namespace hpss {

// Candidate grid, first parameter slowest (buildParameterArrayFor*,
// cmp/linear_search.cu:4-17, zocrs/linear_search.cu:4-34,
// oct/linear_search.cu:4-28).
//  mode 0 (reference): value = lo + idx * inc (one fused multiply-add, as the
//    reference's compiled kernels round it); the velocity is stored as 4/v^2
//    (fast-math division, as the reference computes it on the device).
//  mode 1 (inclusive): both bounds included; the velocity parameter is
//    uniform in c = 4/v^2 from c(lower v) down to c(upper v), the others
//    uniform in value; lo/inc/last arrive as c or value, the last index takes
//    `last` exactly.
struct GridArgs {
    int model, mode;
    float lo[3], inc[3], last[3];
    uint32_t g[3];
};

__device__ __forceinline__ float grid_value(const GridArgs &a, int j, uint32_t idx) {
    if (a.mode == kGridInclusive) {
        if (a.g[j] > 1 && idx == a.g[j] - 1) return a.last[j];
        return __fmaf_rn(static_cast<float>(idx), a.inc[j], a.lo[j]);
    }
    const float v = a.lo[j] + static_cast<float>(idx) * a.inc[j];
    return j == 0 ? 4.0f / (v * v) : v;
}

__global__ void build_grid_kernel(GridArgs a, float *params, uint32_t P) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    if (a.model == kModelCmp) {
        params[i] = grid_value(a, 0, i);
    } else if (a.model == kModelZocrs) {
        const uint32_t iv = (i / (a.g[1] * a.g[2])) % a.g[0];
        const uint32_t ia = (i / a.g[2]) % a.g[1];
        const uint32_t ib = i % a.g[2];
        params[3 * i] = grid_value(a, 0, iv);
        params[3 * i + 1] = grid_value(a, 1, ia);
        params[3 * i + 2] = grid_value(a, 2, ib);
    } else {
        const uint32_t iv = (i / a.g[1]) % a.g[0];
        const uint32_t is = i % a.g[1];
        params[2 * i] = grid_value(a, 0, iv);
        params[2 * i + 1] = grid_value(a, 1, is);
    }
}

cudaError_t launch_build_grid(int model, int mode, const float *lower, const float *inc,
                              const float *last, const uint32_t *gran, float *params,
                              uint32_t P, cudaStream_t st) {
    GridArgs a;
    a.model = model;
    a.mode = mode;
    for (int j = 0; j < 3; j++) {
        a.lo[j] = lower[j];
        a.inc[j] = inc[j];
        a.last[j] = last ? last[j] : 0.f;
        a.g[j] = gran[j];
    }
    uint32_t blocks = (P + 255) / 256;
    build_grid_kernel<<<blocks, 256, 0, st>>>(a, params, P);
    return cudaGetLastError();
}

// Min / max of every parameter over each chunk of `chunkSize` consecutive
// candidates: bounds[k][2*j] = min, bounds[k][2*j+1] = max.
__global__ void chunk_bounds_kernel(const float *params, uint32_t P, int np,
                                    uint32_t chunkSize, uint32_t nChunks,
                                    float *bounds) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nChunks) return;
    uint32_t p0 = k * chunkSize;
    uint32_t p1 = min(P, p0 + chunkSize);
    for (int j = 0; j < np; j++) {
        float lo = INFINITY, hi = -INFINITY;
        for (uint32_t p = p0; p < p1; p++) {
            float v = params[(size_t)p * np + j];
            lo = fminf(lo, v);
            hi = fmaxf(hi, v);
        }
        bounds[(size_t)k * 2 * np + 2 * j] = lo;
        bounds[(size_t)k * 2 * np + 2 * j + 1] = hi;
    }
}

cudaError_t launch_chunk_bounds(const LsParams &p, float *bounds,
                                cudaStream_t st) {
    uint32_t blocks = (p.nChunks + 127) / 128;
    chunk_bounds_kernel<<<blocks, 128, 0, st>>>(p.params, p.P, p.np,
                                                p.chunkSize, p.nChunks, bounds);
    return cudaGetLastError();
}

// OCT trace selection (oct/linear_search.cu:155-192): a trace is used for m0
// if some (t0 sample, sampled candidate) gives a valid displaced midpoint
// within apm of the trace's midpoint.  candFirst/candCount: per-midpoint
// range of traces that can pass at all (|m - m0| <= apm + sqrt(h^2 + h0^2),
// prefiltered on the host); a.selFirst: exclusive prefix of candCount, the
// midpoint's slots in selIdx.
//
// Pass 1: one warp per (midpoint, candidate trace) slot over the whole GPU
// (a trace that is not selected runs every sample and candidate, so the
// slots are spread over all SMs rather than one CTA per midpoint), lanes
// over the sampled candidates, early exit on the first hit; the 0 / 1 flag
// goes to the slot in selIdx.
//
// Lanes first take 32 samples at a time through the box test of all sampled
// candidates at that t0 (oct_sample_may_pass; candBox = their slope and c
// ranges): only samples the box cannot rule out go through the
// per-candidate tests, so a trace that is not selected costs one box test
// per sample instead of one test per (sample, candidate).  The flags are
// those of the per-candidate tests.
__global__ void select_oct_flags_kernel(LsParams a, const float *cands, uint32_t nCand,
                                        const uint32_t *candFirst, uint64_t total,
                                        uint32_t *selIdx, float4 candBox) {
    const int lane = threadIdx.x & 31;
    const uint64_t g = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (g >= total) return;  // whole warps
    // the slot's midpoint: the last mi with selFirst[mi] <= g (midpoints
    // without candidates share their successor's offset)
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
    const float m = a.mid[ti], h = a.hoff[ti];
    const float4 tf = __ldg(ol.tab + ti);
    bool used = false;
    for (uint32_t s0 = 0; s0 < a.S && !used; s0 += 32) {
        const uint32_t sl = s0 + lane;
        // (HPSS_OCT_BOX_TEST=0 turns the box test off: every sample tested)
        const bool may = sl < a.S &&
                         (!a.octBox ||
                          oct_sample_may_pass(tf, h, h0, static_cast<float>(sl) * a.dt,
                                              candBox.x, candBox.y, candBox.z, candBox.w, m0,
                                              a.apm));
        for (uint32_t mask = __ballot_sync(0xffffffffu, may); mask && !used;
             mask &= mask - 1) {
            const float t0 = static_cast<float>(s0 + __ffs(mask) - 1) * a.dt;
            for (uint32_t p0 = 0; p0 < nCand && !used; p0 += 32) {
                const uint32_t p = p0 + lane;
                bool hit = false;
                if (p < nCand) {
                    float mh;
                    const int e = oct_displaced_midpoint(h, h0, t0, m0, cands[2 * p],
                                                         cands[2 * p + 1], &mh);
                    hit = (e == DE_OK && fabsf(m - mh) <= a.apm);
                }
                used = __any_sync(0xffffffffu, hit);
            }
        }
    }
    if (lane == 0) selIdx[g] = used ? 1u : 0u;
}

// Pass 2: order-preserving compaction of every midpoint's flags into its
// selected trace indices, in place: the flags of a chunk of 256 slots are
// all read before any index of the chunk is written, and an index lands at
// or before its flag's slot, never in a later chunk.
constexpr int kCompactThreads = 256;
__global__ void __launch_bounds__(kCompactThreads)
select_oct_compact_kernel(LsParams a, const uint32_t *candFirst, const uint32_t *candCount,
                          uint32_t *selIdx, uint32_t *selCount) {
    const uint32_t mi = blockIdx.x;
    const uint32_t base = a.selFirst[mi], count = candCount[mi], first = candFirst[mi];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kWarps = kCompactThreads / 32;
    __shared__ uint32_t shWarp[kWarps];
    uint32_t done = 0;
    for (uint32_t c = 0; c < count; c += kCompactThreads) {
        const uint32_t q = c + threadIdx.x;
        const bool f = q < count && selIdx[base + q] != 0u;
        const uint32_t bal = __ballot_sync(0xffffffffu, f);
        if (lane == 0) shWarp[warp] = (uint32_t)__popc(bal);
        __syncthreads();  // every flag of the chunk read
        uint32_t before = done, chunk = 0;
        for (int w = 0; w < kWarps; w++) {
            if (w < warp) before += shWarp[w];
            chunk += shWarp[w];
        }
        before += (uint32_t)__popc(bal & ((1u << lane) - 1u));
        if (f) selIdx[base + before] = first + q;
        done += chunk;
        __syncthreads();  // shWarp read by every thread before the next chunk
    }
    if (threadIdx.x == 0) selCount[mi] = done;
}

cudaError_t launch_select_oct(const LsParams &p, const float *cands,
                              uint32_t nCand, uint32_t *selIdx,
                              uint32_t *selCount, const uint32_t *candFirst,
                              const uint32_t *candCount, uint64_t total, float4 candBox,
                              cudaStream_t st) {
    if (p.nM0 == 0) return cudaSuccess;
    if (total > 0) {
        const uint64_t blocks = (total * 32 + 255) / 256;
        if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
        select_oct_flags_kernel<<<(uint32_t)blocks, 256, 0, st>>>(p, cands, nCand, candFirst,
                                                                  total, selIdx, candBox);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return launch_select_compact(p, candFirst, candCount, selIdx, selCount, st);
}

cudaError_t launch_select_compact(const LsParams &p, const uint32_t *candFirst,
                                  const uint32_t *candCount, uint32_t *selIdx,
                                  uint32_t *selCount, cudaStream_t st) {
    if (p.nM0 == 0) return cudaSuccess;
    select_oct_compact_kernel<<<p.nM0, kCompactThreads, 0, st>>>(p, candFirst, candCount,
                                                                  selIdx, selCount);
    return cudaGetLastError();
}

// FP32 -> BF16 / FP16 (+ per-trace scale for FP16) storage conversion.
__global__ void convert_storage_kernel(const float *src, uint16_t *dst,
                                       float *scale, uint32_t nTraces,
                                       uint32_t S, uint32_t stride,
                                       int storage) {
    uint32_t tr = blockIdx.x;
    if (tr >= nTraces) return;
    const float *row = src + (size_t)tr * stride;
    __shared__ float shMax[32];
    float mx = 0.f;
    for (uint32_t i = threadIdx.x; i < S; i += blockDim.x)
        mx = fmaxf(mx, fabsf(row[i]));
    for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) shMax[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? shMax[threadIdx.x] : 0.f;
        for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) shMax[0] = v;
    }
    __syncthreads();
    // FP16: scale the trace so its peak maps to 2^14 (inside FP16 range with
    // headroom); the kernel multiplies back by scale.
    float sc = 1.f;
    if (storage == 2) {
        float peak = shMax[0];
        sc = peak > 0.f ? peak / 16384.f : 1.f;
        if (threadIdx.x == 0) scale[tr] = sc;
    } else if (threadIdx.x == 0 && scale) {
        scale[tr] = 1.f;
    }
    float inv = 1.f / sc;
    uint16_t *out = dst + (size_t)tr * stride;
    for (uint32_t i = threadIdx.x; i < stride; i += blockDim.x) {
        float v = i < S ? row[i] : 0.f;
        uint16_t bits;
        if (storage == 1) {
            __nv_bfloat16 b = __float2bfloat16_rn(v);
            bits = *reinterpret_cast<uint16_t *>(&b);
        } else {
            __half hv = __float2half_rn(v * inv);
            bits = *reinterpret_cast<uint16_t *>(&hv);
        }
        out[i] = bits;
    }
}

cudaError_t launch_convert_storage(const float *src, uint16_t *dst,
                                   float *scale, uint32_t nTraces, uint32_t S,
                                   uint32_t stride, int storage,
                                   cudaStream_t st) {
    if (nTraces == 0) return cudaSuccess;
    convert_storage_kernel<<<nTraces, 256, 0, st>>>(src, dst, scale, nTraces,
                                                    S, stride, storage);
    return cudaGetLastError();
}

}  // namespace hpss
