// noalloc.cu -- linear search for callers that cannot allocate device memory.
//
// Some hosts of this library may not call cudaMalloc: a plug-in running inside
// another framework's memory pool, a process with a fixed device-memory
// budget negotiated up front, or code that must not allocate after start-up.
// hpss_linear_search_noalloc serves them: the caller passes its own device
// buffers for inputs and output, and the scratch the search needs (candidate
// grid, per-chunk bounds, squared half-offsets, per-midpoint trace ranges,
// error word) lives in one file-scope __device__ array of fixed size below.
// Every GPU that loads the library holds that array until the process exits.
//
// The array's name in host code is only a host-side stand-in, not a device
// address: the address is looked up with cudaGetSymbolAddress once per
// device, with that device current, on the first call made on that device
// (so make that first call before any stream capture).  All calls share the
// one array and it keeps the previous call's contents: this file clears what
// must start at zero on every call, and calls whose work overlaps on the GPU
// (different streams, or different host threads on the same device) race on
// it -- serialise them.  The kernels' device error word is part of that
// array too: hpss_noalloc_device_error reads it once the call has finished.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/hpss.h"
#include "hpss_internal.h"

namespace hpss {
cudaError_t launch_select_range(const float *mid, uint32_t n, const float *m0s,
                                uint32_t nM0, int mode, float apm, float radius,
                                uint32_t *first, uint32_t *count, cudaStream_t st);
size_t tuned_stage_floats();
void set_thread_error(const std::string &msg);
}  // namespace hpss

using namespace hpss;

namespace {

// Limits of the allocation-free entry point (the scratch is sized for them).
constexpr uint32_t kNaMaxCandidates = 65536;
constexpr uint32_t kNaMaxMidpoints = 16384;
constexpr uint32_t kNaMaxTraces = 1u << 20;
constexpr uint32_t kNaChunk = kTunedWarps * 4;  // tuned kernel, 2 pairs per thread

// scratch layout, in 4-byte words, each region 256-byte aligned
constexpr size_t align64(size_t w) { return (w + 63) & ~size_t(63); }
constexpr size_t kOffParams = 0;
constexpr size_t kOffBounds = kOffParams + align64((size_t)kNaMaxCandidates * 3);
constexpr size_t kOffHsq = kOffBounds + align64((size_t)(kNaMaxCandidates / kNaChunk + 1) * 6);
constexpr size_t kOffFirst = kOffHsq + align64(kNaMaxTraces);
constexpr size_t kOffCount = kOffFirst + align64(kNaMaxMidpoints);
constexpr size_t kOffErr = kOffCount + align64(kNaMaxMidpoints);
constexpr size_t kScratchWords = kOffErr + 64;

// ~5.3 MB per device
__device__ __align__(256) uint32_t g_noallocScratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratchAddr[kMaxDevices] = {};

hpss_status fail(hpss_status code, const std::string &msg) {
    set_thread_error(msg);  // read back with hpss_last_error(NULL)
    return code;
}

// Device address of the scratch array on the current device, looked up
// once per device with that device current (the array's name in host code is
// only a host-side stand-in).  The address is kept for the life of the
// process: it is not valid across cudaDeviceReset, after which this library
// must not be called again on that device.
hpss_status scratch_of_current_device(int *devOut, void **base) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(HPSS_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(HPSS_ERR_NO_DEVICE, "device index too large");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratchAddr[dev]) {
        e = cudaGetSymbolAddress(&g_scratchAddr[dev], g_noallocScratch);
        if (e != cudaSuccess) {
            g_scratchAddr[dev] = nullptr;
            return fail(HPSS_ERR_CUDA,
                        std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        }
    }
    *devOut = dev;
    *base = g_scratchAddr[dev];
    return HPSS_OK;
}

__global__ void square_kernel(const float *h, float *hsq, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) hsq[i] = h[i] * h[i];  // float h*h, as the reference's host code
}

}  // namespace

extern "C" hpss_status hpss_linear_search_noalloc(
    int model, const float *d_samples, uint32_t stride, const float *d_midpoints,
    const float *d_halfoffsets, uint32_t nTraces, uint32_t samplesPerTrace, float dtInSeconds,
    int tauIndexDisplacement, const float *lower, const float *upper,
    const uint32_t *granularity, float apm, const float *d_m0s, uint32_t nM0, float *d_out,
    void *stream) {
    if (model != HPSS_MODEL_CMP && model != HPSS_MODEL_ZOCRS)
        return fail(HPSS_ERR_INVALID_ARGUMENT, "allocation-free search supports CMP and ZO-CRS");
    const int np = model == HPSS_MODEL_CMP ? 1 : 3;
    if (!lower || !upper || !granularity)
        return fail(HPSS_ERR_LOGIC, "bounds and granularity are required");
    if (nM0 == 0) return HPSS_OK;
    if (!d_samples || !d_midpoints || !d_halfoffsets || !d_m0s || !d_out)
        return fail(HPSS_ERR_INVALID_ARGUMENT, "null device pointer");
    if (samplesPerTrace == 0 || !(dtInSeconds > 0.f) || stride < samplesPerTrace ||
        stride % 4 != 0 || (reinterpret_cast<uintptr_t>(d_samples) & 15) != 0)
        return fail(HPSS_ERR_INVALID_ARGUMENT,
                    "need S > 0, dt > 0, stride >= S, stride % 4 == 0, 16-byte aligned samples");
    if (tauIndexDisplacement < 0 || 2 * tauIndexDisplacement + 1 > kMaxWindow)
        return fail(HPSS_ERR_INVALID_ARGUMENT, "window 2*tau+1 must be in [1, 31]");
    uint64_t P = 1;
    uint32_t gran[3] = {1, 1, 1};
    float inc[3] = {0, 0, 0}, low[3] = {0, 0, 0};
    for (int j = 0; j < np; j++) {
        if (granularity[j] == 0) return fail(HPSS_ERR_INVALID_ARGUMENT, "granularity must be > 0");
        gran[j] = granularity[j];
        P *= granularity[j];
        low[j] = lower[j];
        inc[j] = (upper[j] - lower[j]) / static_cast<float>(granularity[j]);
    }
    if (P > kNaMaxCandidates || nM0 > kNaMaxMidpoints || nTraces > kNaMaxTraces)
        return fail(HPSS_ERR_INVALID_ARGUMENT,
                    "allocation-free search limits: candidates <= 65536, midpoints <= 16384, "
                    "traces <= 1048576");

    int dev = 0;
    void *base = nullptr;
    hpss_status rc = scratch_of_current_device(&dev, &base);
    if (rc != HPSS_OK) return rc;
    cudaError_t e = cudaSuccess;
    uint32_t *w = static_cast<uint32_t *>(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    LsParams lp{};
    lp.samples = d_samples;
    lp.stride = stride;
    lp.S = samplesPerTrace;
    lp.dt = dtInSeconds;
    lp.tau = tauIndexDisplacement;
    lp.w = 2 * tauIndexDisplacement + 1;
    lp.mid = d_midpoints;
    lp.hoff = d_halfoffsets;
    lp.hsq = reinterpret_cast<float *>(w + kOffHsq);
    lp.m0s = d_m0s;
    lp.nM0 = nM0;
    lp.params = reinterpret_cast<float *>(w + kOffParams);
    lp.P = (uint32_t)P;
    lp.np = np;
    lp.chunkSize = kNaChunk;
    lp.nChunks = (lp.P + kNaChunk - 1) / kNaChunk;
    lp.chunkBounds = reinterpret_cast<float *>(w + kOffBounds);
    lp.apm = apm;
    lp.selFirst = w + kOffFirst;
    lp.selCount = w + kOffCount;
    lp.out = d_out;
    lp.errorWord = w + kOffErr;
    set_stage_drill(lp);

    // the error word keeps the previous call's value: clear it
    e = cudaMemsetAsync(lp.errorWord, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess && nTraces)
        square_kernel<<<(nTraces + 255) / 256, 256, 0, st>>>(d_halfoffsets,
                                                              reinterpret_cast<float *>(w + kOffHsq),
                                                              nTraces);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess)
        e = launch_build_grid(model, kGridReference, low, inc, nullptr, gran,
                              reinterpret_cast<float *>(w + kOffParams), lp.P, st);
    if (e == cudaSuccess)
        e = launch_chunk_bounds(lp, reinterpret_cast<float *>(w + kOffBounds), st);
    if (e == cudaSuccess)
        e = launch_select_range(d_midpoints, nTraces, d_m0s, nM0,
                                model == HPSS_MODEL_CMP ? 0 : 1, apm, 0.f, w + kOffFirst,
                                w + kOffCount, st);
    if (e != cudaSuccess) return fail(HPSS_ERR_CUDA, cudaGetErrorString(e));

    const bool tuned = lp.w <= 15 && stride + 8 <= (uint32_t)tuned_stage_floats();
    if (tuned) {
        const uint32_t tiles = (samplesPerTrace + kTileSamples - 1) / kTileSamples;
        const uint64_t units = (uint64_t)nM0 * tiles;
        int sms = 1;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const uint32_t grid = (uint32_t)std::min<uint64_t>(units, (uint64_t)sms * 2);
        e = model == HPSS_MODEL_CMP
                ? launch_ls_tuned_cmp(lp, grid, tiles, (uint32_t)units, st, 0, false)
                : launch_ls_tuned_zocrs(lp, grid, tiles, (uint32_t)units, st, 0, false);
    } else {
        e = launch_ls_plain(lp, st);
    }
    if (e != cudaSuccess) return fail(HPSS_ERR_CUDA, cudaGetErrorString(e));
    return HPSS_OK;
}

// The allocating entry points report the kernels' device error word in
// hpss_stats.device_error; the allocation-free search is asynchronous and has
// no statistics, so its word (it lives in the shared scratch array) is read
// here: after the stream has finished the call, one 4-byte copy to the
// caller's host variable.  No allocation.
extern "C" hpss_status hpss_noalloc_device_error(void *stream, uint32_t *word) {
    if (!word) return fail(HPSS_ERR_INVALID_ARGUMENT, "null output pointer");
    int dev = 0;
    void *base = nullptr;
    hpss_status rc = scratch_of_current_device(&dev, &base);
    if (rc != HPSS_OK) return rc;
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess)
        e = cudaMemcpy(word, static_cast<uint32_t *>(base) + kOffErr, sizeof(uint32_t),
                       cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(HPSS_ERR_CUDA, cudaGetErrorString(e));
    return HPSS_OK;
}
