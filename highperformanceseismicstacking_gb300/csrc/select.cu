// select.cu -- trace selection for a batch of midpoints, on the device.
//
// The line is resident and sorted by (midpoint, half-offset), so the
// reference's per-midpoint mask kernels (cmp/common.cu:3-15: m == m0;
// zocrs/common.cu:3-16: |m0 - m| <= apm) select one contiguous run of traces:
// a binary search per midpoint with the reference's own predicate finds it,
// and no trace is copied (the reference packs the selected traces with one
// cudaMemcpy per trace, ComputeAlgorithm.cpp:107-153).
#include "hpss_device.cuh"
#include "hpss_internal.h"

namespace hpss {

// first index in [0, n) where pred(i) is true, for a predicate that is
// false...false true...true over the sorted midpoints
template <typename Pred>
__device__ __forceinline__ uint32_t lower_bound_pred(uint32_t n, Pred pred) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = lo + ((hi - lo) >> 1);
        if (pred(mid)) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// mode 0: CMP equality; mode 1: ZO-CRS |m0 - m| <= apm; mode 2: OCT candidate
// range |m0 - m| <= radius (prefilter; the exact test follows).
__global__ void select_range_kernel(const float *mid, uint32_t n,
                                    const float *m0s, uint32_t nM0, int mode,
                                    float apm, float radius, uint32_t *first,
                                    uint32_t *count) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nM0) return;
    const float m0 = m0s[i];
    uint32_t a, b;
    if (mode == 0) {
        a = lower_bound_pred(n, [&](uint32_t j) { return mid[j] >= m0; });
        b = lower_bound_pred(n, [&](uint32_t j) { return mid[j] > m0; });
        // the reference predicate is m0 == m: equal floats only
        if (!(m0 == m0)) b = a;
    } else {
        const float r = mode == 1 ? apm : radius;
        a = lower_bound_pred(n, [&](uint32_t j) {
            float m = mid[j];
            return m >= m0 || fabsf(m0 - m) <= r;
        });
        b = lower_bound_pred(n, [&](uint32_t j) {
            float m = mid[j];
            return m > m0 && !(fabsf(m0 - m) <= r);
        });
        if (b < a) b = a;
    }
    first[i] = a;
    count[i] = b - a;
}

// Midpoints in descending order of selected traces (ties by index):
// order[rank(i)] = i with rank(i) = #{j : count[j] > count[i] or
// (count[j] == count[i] and j < i)}.  Quadratic, for up to a few thousand
// midpoints (the host sorts only batches up to kMaxOrderedMidpoints).
__global__ void order_by_count_kernel(const uint32_t *count, uint32_t n, uint32_t *order) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t ci = count[i];
    uint32_t rank = 0;
    for (uint32_t j = 0; j < n; j++) {
        const uint32_t cj = count[j];
        rank += (cj > ci || (cj == ci && j < i)) ? 1u : 0u;
    }
    order[rank] = i;
}

cudaError_t launch_order_by_count(const uint32_t *count, uint32_t n, uint32_t *order,
                                  cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    order_by_count_kernel<<<(n + 255) / 256, 256, 0, st>>>(count, n, order);
    return cudaGetLastError();
}

// exclusive prefix sum of count[] into first[] (single CTA, any n)
__global__ void exclusive_scan_kernel(const uint32_t *count, uint32_t *first,
                                      uint32_t n) {
    __shared__ uint32_t warpSums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < n ? count[i] : 0;
        uint32_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warpSums[warp] = incl;
        __syncthreads();
        uint32_t woff = 0;
        for (int w = 0; w < warp; w++) woff += warpSums[w];
        if (i < n) first[i] = carry + woff + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += woff + incl;
        __syncthreads();
    }
}

cudaError_t launch_select_range(const float *mid, uint32_t n, const float *m0s,
                                uint32_t nM0, int mode, float apm, float radius,
                                uint32_t *first, uint32_t *count,
                                cudaStream_t st) {
    if (nM0 == 0) return cudaSuccess;
    select_range_kernel<<<(nM0 + 127) / 128, 128, 0, st>>>(
        mid, n, m0s, nM0, mode, apm, radius, first, count);
    return cudaGetLastError();
}

cudaError_t launch_exclusive_scan(const uint32_t *count, uint32_t *first,
                                  uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    exclusive_scan_kernel<<<1, 1024, 0, st>>>(count, first, n);
    return cudaGetLastError();
}

}  // namespace hpss
