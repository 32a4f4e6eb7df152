// hpss_capi.cu -- the C ABI of libhpss_gb300.so (declared in include/hpss.h):
// handle lifecycle, the resident line, the setters and the extern "C" entry
// points (the linear search and DE host logic are in ls_host.cu / de_host.cu).
//
// Host-side orchestration only: argument checks with the reference's error
// semantics, device buffers owned by the handle, and the launch sequence
// (candidate grid -> trace selection -> semblance kernel) on the handle's
// stream.  No exception crosses the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "hpss_handle.h"

using namespace hpss;


namespace {
thread_local std::string g_createError;
const char *kVersion = "hpss-gb300 0.1.0 (sm_103a)";
}  // namespace

namespace hpss {

struct Fail {
    hpss_status code;
};

hpss_status set_error(hpss_handle h, hpss_status code, const std::string &msg) {
    if (h) h->lastError = msg;
    else g_createError = msg;
    return code;
}


cudaError_t ensure(hpss_handle h, hpss_handle_s::Buf &b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return cudaSuccess;
    if (b.p) {
        cudaFree(b.p);
        h->deviceBytes -= b.bytes;
        b.p = nullptr;
        b.bytes = 0;
    }
    size_t want = std::max(bytes, (size_t)256);
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) return e;
    b.bytes = want;
    h->deviceBytes += want;
    return cudaSuccess;
}

void release(hpss_handle h, hpss_handle_s::Buf &b) {
    if (b.p) {
        cudaFree(b.p);
        h->deviceBytes -= b.bytes;
    }
    b.p = nullptr;
    b.bytes = 0;
}

void free_gather(hpss_handle h) {
    auto fr = [&](void *&p, size_t bytes) {
        if (p) {
            cudaFree(p);
            h->deviceBytes -= bytes;
        }
        p = nullptr;
    };
    fr(reinterpret_cast<void *&>(h->dSamples), h->capSamples);
    fr(reinterpret_cast<void *&>(h->dSamples16), h->capSamples16);
    fr(h->dTraceBuf, h->capTrace);
    h->dScale = h->dMid = h->dHoff = h->dHsq = nullptr;
    h->capSamples = h->capSamples16 = h->capTrace = 0;
    h->gatherReady = false;
    h->octTabValid = false;
}

// Line buffer of at least `bytes`: the current allocation when it is large
// enough (a re-upload of a line of the same size allocates nothing), else a
// new one.
cudaError_t grow_line_buffer(hpss_handle h, void **p, size_t &cap, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (*p && cap >= bytes) return cudaSuccess;
    if (*p) {
        cudaFree(*p);
        h->deviceBytes -= cap;
        *p = nullptr;
        cap = 0;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return e;
    cap = bytes;
    h->deviceBytes += bytes;
    return cudaSuccess;
}

int model_params(int model) {
    return model == HPSS_MODEL_CMP ? 1 : (model == HPSS_MODEL_ZOCRS ? 3 : 2);
}

hpss_status check_ready(hpss_handle h) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (!h->gatherReady)
        return set_error(h, HPSS_ERR_NOT_READY, "no gather uploaded (hpss_upload_gather)");
    if (h->model < 0)
        return set_error(h, HPSS_ERR_NOT_READY, "no traveltime model set (hpss_set_traveltime)");
    if (h->tau < 0)
        return set_error(h, HPSS_ERR_NOT_READY, "no semblance window set (hpss_set_window)");
    return HPSS_OK;
}

// The 1024 sampled OCT candidates of the reference's linear-search trace
// selection (CudaLinearSearchAlgorithm.cu:269-292): a default-constructed
// std::default_random_engine, one uniform_real_distribution<float> per
// parameter over [lower, upper); velocity converted to 4/v^2 on the host.
void build_oct_selection_candidates(hpss_handle h) {
    const unsigned samplePop = 1024;
    h->octCandsHost.assign(samplePop * 2, 0.f);
    std::default_random_engine generator;
    for (unsigned prm = 0; prm < 2; prm++) {
        std::uniform_real_distribution<float> dist(h->lower[prm], h->upper[prm]);
        for (unsigned i = 0; i < samplePop; i++) {
            float v = dist(generator);
            if (prm == 0) v = 4.0f / (v * v);
            h->octCandsHost[i * 2 + prm] = v;
        }
    }
}

// OCT selection, the step shared by the linear search, DE and stretch-free:
// only traces with |m - m0| <= apm + sqrt(hmax^2 + h0^2) can pass (the
// displaced midpoint formula, oct/common.cuh:26-32, divides
// 2*theta*(h^2-h0^2) by a root no smaller than 2*|theta|*sqrt(h^2+h0^2)),
// widened for rounding: a contiguous run of the sorted line per midpoint
// (candFirst / candCount).  Each midpoint gets that many slots of selIdx, at
// offsets `first` (exclusive prefix sum, 32-bit: a total of 2^32 slots or
// more is rejected); selIdx is grown to the total.
hpss_status oct_candidate_slots(hpss_handle h, const float *d_m0s, uint32_t nM0,
                                uint32_t *first, uint64_t *total) {
    float hmax = 0.f, h0max = std::fabs(h->h0);
    for (float v : h->hHoff) hmax = std::max(hmax, std::fabs(v));
    for (float v : h->octH0s) h0max = std::max(h0max, std::fabs(v));
    float radius = (h->apm + std::sqrt(hmax * hmax + h0max * h0max)) * 1.001f + 1.0f;
    HPSS_CUDA_TRY(h, ensure(h, h->candFirst, nM0 * sizeof(uint32_t)));
    HPSS_CUDA_TRY(h, ensure(h, h->candCount, nM0 * sizeof(uint32_t)));
    uint32_t *cf = static_cast<uint32_t *>(h->candFirst.p);
    uint32_t *cc = static_cast<uint32_t *>(h->candCount.p);
    HPSS_CUDA_TRY(h, launch_select_range(h->dMid, h->nTraces, d_m0s, nM0, 2,
                                         h->apm, radius, cf, cc, h->stream));
    HPSS_CUDA_TRY(h, launch_exclusive_scan(cc, first, nM0, h->stream));
    std::vector<uint32_t> ccHost(nM0);
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(ccHost.data(), cc, nM0 * sizeof(uint32_t),
                                     cudaMemcpyDeviceToHost, h->stream));
    HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    uint64_t t = 0;
    for (uint32_t v : ccHost) t += v;
    if (t > 0xffffffffull)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT,
                         "OCT selection: 2^32 or more candidate trace slots in one call; "
                         "split the midpoints into smaller calls");
    HPSS_CUDA_TRY(h, ensure(h, h->selIdx, t * sizeof(uint32_t)));
    *total = t;
    return HPSS_OK;
}

// Device-side selection for nM0 midpoints (d_m0s on the device).  Leaves
// LsParams' selFirst / selCount / selIdx filled.
hpss_status run_selection(hpss_handle h, const float *d_m0s, uint32_t nM0,
                          LsParams &lp) {
    HPSS_CUDA_TRY(h, ensure(h, h->selFirst, nM0 * sizeof(uint32_t)));
    HPSS_CUDA_TRY(h, ensure(h, h->selCount, nM0 * sizeof(uint32_t)));
    uint32_t *first = static_cast<uint32_t *>(h->selFirst.p);
    uint32_t *count = static_cast<uint32_t *>(h->selCount.p);
    lp.selFirst = first;
    lp.selCount = count;
    lp.selIdx = nullptr;
    if (h->model != HPSS_MODEL_OCT) {
        HPSS_CUDA_TRY(h, launch_select_range(h->dMid, h->nTraces, d_m0s, nM0,
                                             h->model == HPSS_MODEL_CMP ? 0 : 1,
                                             h->apm, 0.f, first, count, h->stream));
        return HPSS_OK;
    }
    uint64_t total = 0;
    hpss_status rc = oct_candidate_slots(h, d_m0s, nM0, first, &total);
    if (rc != HPSS_OK) return rc;
    const uint32_t *cf = static_cast<const uint32_t *>(h->candFirst.p);
    const uint32_t *cc = static_cast<const uint32_t *>(h->candCount.p);
    if (h->octCandsHost.empty()) build_oct_selection_candidates(h);
    HPSS_CUDA_TRY(h, ensure(h, h->octCands, h->octCandsHost.size() * sizeof(float)));
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(h->octCands.p, h->octCandsHost.data(),
                                     h->octCandsHost.size() * sizeof(float),
                                     cudaMemcpyHostToDevice, h->stream));
    lp.selIdx = static_cast<uint32_t *>(h->selIdx.p);
    lp.m0s = d_m0s;
    lp.nM0 = nM0;
    // slope and c ranges of the sampled candidates (the selection's box test)
    float4 box = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
    for (size_t i = 0; i + 1 < h->octCandsHost.size(); i += 2) {
        box.z = std::min(box.z, h->octCandsHost[i]);
        box.w = std::max(box.w, h->octCandsHost[i]);
        box.x = std::min(box.x, h->octCandsHost[i + 1]);
        box.y = std::max(box.y, h->octCandsHost[i + 1]);
    }
    HPSS_CUDA_TRY(h, use_oct_table(h, lp));
    HPSS_CUDA_TRY(h, launch_select_oct(lp, static_cast<const float *>(h->octCands.p),
                                       (uint32_t)(h->octCandsHost.size() / 2),
                                       static_cast<uint32_t *>(h->selIdx.p), count,
                                       cf, cc, (uint64_t)total, box, h->stream));
    return HPSS_OK;
}

void fill_line_params(hpss_handle h, LsParams &lp) {
    lp = LsParams{};
    // the line is resident in one storage only: FP32 rows, or 16-bit rows
    // (every kernel widens them as it reads; dSamples is then only the
    // upload's FP32 staging area)
    lp.samples = h->storage == HPSS_STORAGE_FP32 ? h->dSamples : nullptr;
    lp.samples16 = h->storage != HPSS_STORAGE_FP32 ? h->dSamples16 : nullptr;
    lp.scale = h->storage != HPSS_STORAGE_FP32 ? h->dScale : nullptr;
    lp.storage = h->storage;
    lp.stride = h->stride;
    lp.S = h->S;
    lp.dt = h->dt;
    lp.tau = h->tau;
    lp.w = 2 * h->tau + 1;
    lp.mid = h->dMid;
    lp.hoff = h->dHoff;
    lp.hsq = h->dHsq;
    lp.np = (int)h->np;
    lp.apm = h->apm;
    lp.h0 = h->h0;
}

// OCT: the per-trace factor tables of the resident line -- one for the
// current h0, or one per target half-offset of hpss_set_oct_half_offsets,
// octTabStride entries apart -- built on the handle's stream at the first OCT
// call after an upload or a change of the half-offsets.
cudaError_t use_oct_table(hpss_handle h, LsParams &lp) {
    if (h->model != HPSS_MODEL_OCT) return cudaSuccess;
    const std::vector<float> want = h->octH0s.empty() ? std::vector<float>{h->h0} : h->octH0s;
    if (!h->octTabValid || h->octTabH0s != want) {
        h->octTabValid = false;
        cudaError_t e = ensure(h, h->octTab, want.size() * (size_t)h->nTraces * sizeof(float4));
        if (e != cudaSuccess) return e;
        for (size_t b = 0; b < want.size(); b++) {
            e = launch_oct_trace_table(h->dMid, h->dHoff, h->nTraces, want[b],
                                       static_cast<float4 *>(h->octTab.p) + b * h->nTraces,
                                       h->stream);
            if (e != cudaSuccess) return e;
        }
        h->octTabValid = true;
        h->octTabH0s = want;
    }
    lp.octTab = static_cast<const float4 *>(h->octTab.p);
    lp.octTabStride = h->nTraces;
    // HPSS_OCT_BOX_TEST=0 turns the displaced-midpoint box test off (every
    // trace through the per-sample test; same results, for A/B checks)
    const char *box = std::getenv("HPSS_OCT_BOX_TEST");
    lp.octBox = !(box && box[0] == '0');
    return cudaSuccess;
}

uint32_t h0_blocks(hpss_handle h) {
    return h->model == HPSS_MODEL_OCT && !h->octH0s.empty() ? (uint32_t)h->octH0s.size() : 1u;
}

cudaError_t expand_h0_blocks(hpss_handle h, LsParams &lp) {
    const uint32_t nb = h0_blocks(h);
    if (nb == 1 || lp.nM0 == 0) return cudaSuccess;
    const uint32_t n = lp.nM0;
    cudaError_t e = ensure(h, h->m0v, (size_t)nb * n * sizeof(float));
    if (e != cudaSuccess) return e;
    float *dst = static_cast<float *>(h->m0v.p);
    for (uint32_t b = 0; b < nb; b++) {
        e = cudaMemcpyAsync(dst + (size_t)b * n, lp.m0s, n * sizeof(float),
                            cudaMemcpyDeviceToDevice, h->stream);
        if (e != cudaSuccess) return e;
    }
    lp.m0s = dst;
    lp.nM0 = nb * n;
    lp.m0PerH0 = n;
    lp.h0s = static_cast<const float *>(h->octH0sDev.p);
    return cudaSuccess;
}

int num_sms(hpss_handle h) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, h->device);
    return v > 0 ? v : 1;
}

// 16-bit storage: the FP32 staging area of an upload, released once the
// upload's copies and conversions have finished (stream synchronised), so
// no FP32 rows stay resident.
void release_upload_staging(hpss_handle h) {
    if (h->storage == HPSS_STORAGE_FP32 || !h->dSamples) return;
    cudaFree(h->dSamples);
    h->deviceBytes -= h->capSamples;
    h->dSamples = nullptr;
    h->capSamples = 0;
}

// Rows of the FP32 staging area of a 16-bit upload (about 64 MB).
size_t stage_rows(hpss_handle h) {
    constexpr size_t kStageBytes = size_t(64) << 20;
    return std::max<size_t>(1, kStageBytes / ((size_t)h->stride * sizeof(float)));
}

// A new line, everything but the amplitudes: validation, host geometry,
// device buffers (grown as needed) and the geometry copies on the handle's
// stream.  The amplitudes follow with copy_line_rows.
hpss_status prepare_line(hpss_handle h, const float *samples, const float *midpoints,
                         const float *halfoffsets, uint32_t nTraces, uint32_t samplesPerTrace,
                         float dtInSeconds, int storage) {
    if (nTraces > 0 && (!samples || !midpoints || !halfoffsets))
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "null input array");
    if (samplesPerTrace == 0 || !(dtInSeconds > 0.f))
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "samplesPerTrace and dt must be > 0");
    // the tuned kernels take floor(t/dt) through a 2^23 offset add
    if (samplesPerTrace > (1u << 22))
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "samplesPerTrace must be <= 2^22");
    if (storage < HPSS_STORAGE_FP32 || storage > HPSS_STORAGE_FP16)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "unknown storage");
    for (uint32_t i = 0; i < nTraces; i++) {
        float m = midpoints[i], o = halfoffsets[i];
        if (!std::isfinite(m) || !std::isfinite(o))
            return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "non-finite midpoint or half-offset");
        if (i > 0) {
            float pm = midpoints[i - 1], ph = halfoffsets[i - 1];
            if (m < pm || (m == pm && o < ph))
                return set_error(h, HPSS_ERR_INVALID_ARGUMENT,
                                 "traces must be sorted by (midpoint, half-offset)");
        }
    }
    cudaSetDevice(h->device);
    // earlier work may still read the buffers about to be overwritten
    cudaStreamSynchronize(h->stream);
    if (h->copyStream) cudaStreamSynchronize(h->copyStream);
    h->gatherReady = false;
    h->octTabValid = false;
    h->nTraces = nTraces;
    h->S = samplesPerTrace;
    h->stride = (samplesPerTrace + 7u) & ~7u;  // 32-byte rows
    h->dt = dtInSeconds;
    h->storage = storage;
    h->hMid.assign(midpoints, midpoints + nTraces);
    h->hHoff.assign(halfoffsets, halfoffsets + nTraces);
    {
        uint32_t distinct = 0;
        for (uint32_t i = 0; i < nTraces; i++)
            if (i == 0 || midpoints[i] != midpoints[i - 1]) distinct++;
        h->meanFold = distinct ? nTraces / distinct : 0;
    }
    // h*h in float as the reference's host code; kept in the handle while
    // its copy is in flight
    h->hHsq.resize(nTraces);
    for (uint32_t i = 0; i < nTraces; i++) h->hHsq[i] = halfoffsets[i] * halfoffsets[i];
    const size_t n = nTraces, st = h->stride;
    // the line is resident in one storage only: a buffer of the other one
    // left by an earlier line is released (and the FP32 buffer shrunk to the
    // staging area of a 16-bit upload)
    auto release_line_buffer = [&](void **p, size_t &cap) {
        if (*p) {
            cudaFree(*p);
            h->deviceBytes -= cap;
        }
        *p = nullptr;
        cap = 0;
    };
    if (storage == HPSS_STORAGE_FP32) {
        release_line_buffer(reinterpret_cast<void **>(&h->dSamples16), h->capSamples16);
        HPSS_CUDA_TRY(h, grow_line_buffer(h, reinterpret_cast<void **>(&h->dSamples),
                                          h->capSamples, n * st * sizeof(float)));
    } else {
        // 16-bit storage: the line lives in 16-bit rows only; the FP32 rows
        // pass through a staging area of at most about 64 MB on their way,
        // released when the upload is done (release_upload_staging)
        const size_t stageBytes = std::min<size_t>(n, stage_rows(h)) * st * sizeof(float);
        if (h->capSamples > std::max<size_t>(stageBytes, 16))
            release_line_buffer(reinterpret_cast<void **>(&h->dSamples), h->capSamples);
        HPSS_CUDA_TRY(h, grow_line_buffer(h, reinterpret_cast<void **>(&h->dSamples16),
                                          h->capSamples16, n * st * sizeof(uint16_t)));
        HPSS_CUDA_TRY(h, grow_line_buffer(h, reinterpret_cast<void **>(&h->dSamples),
                                          h->capSamples, stageBytes));
    }
    // mid, hoff, hsq and the 16-bit storage scale: four 256-byte aligned
    // slices of one buffer
    const size_t slice = (n * sizeof(float) + 255) & ~size_t(255);
    HPSS_CUDA_TRY(h, grow_line_buffer(h, &h->dTraceBuf, h->capTrace, 4 * slice));
    char *tb = static_cast<char *>(h->dTraceBuf);
    h->dMid = reinterpret_cast<float *>(tb);
    h->dHoff = reinterpret_cast<float *>(tb + slice);
    h->dHsq = reinterpret_cast<float *>(tb + 2 * slice);
    h->dScale = reinterpret_cast<float *>(tb + 3 * slice);
    if (n) {
        HPSS_CUDA_TRY(h, cudaMemcpyAsync(h->dMid, midpoints, n * sizeof(float),
                                         cudaMemcpyHostToDevice, h->stream));
        HPSS_CUDA_TRY(h, cudaMemcpyAsync(h->dHoff, halfoffsets, n * sizeof(float),
                                         cudaMemcpyHostToDevice, h->stream));
        HPSS_CUDA_TRY(h, cudaMemcpyAsync(h->dHsq, h->hHsq.data(), n * sizeof(float),
                                         cudaMemcpyHostToDevice, h->stream));
    }
    return HPSS_OK;
}

// Amplitudes of traces [a, b) on stream st.  FP32 storage: one copy into
// the line when rows need no padding, a pitched copy otherwise (the padding
// is zeroed by the caller).  16-bit storage: pieces of at most stage_rows
// rows are copied into the staging area and converted into the 16-bit line
// (stream order keeps a piece's conversion before the next piece's copy; the
// converter writes the rows' zero padding itself).
cudaError_t copy_line_rows(hpss_handle h, const float *samples, uint32_t a, uint32_t b,
                           cudaStream_t st) {
    if (b <= a) return cudaSuccess;
    const size_t S = h->S, pitch = h->stride;
    auto copyRows = [&](float *dst, uint32_t r0, size_t rows) {
        const float *src = samples + (size_t)r0 * S;
        return pitch == S ? cudaMemcpyAsync(dst, src, rows * S * sizeof(float),
                                            cudaMemcpyHostToDevice, st)
                          : cudaMemcpy2DAsync(dst, pitch * sizeof(float), src, S * sizeof(float),
                                              S * sizeof(float), rows, cudaMemcpyHostToDevice,
                                              st);
    };
    if (h->storage == HPSS_STORAGE_FP32) return copyRows(h->dSamples + (size_t)a * pitch, a, b - a);
    const uint32_t piece = (uint32_t)stage_rows(h);
    for (uint32_t r = a; r < b; r += piece) {
        const uint32_t rows = std::min(piece, b - r);
        cudaError_t e = copyRows(h->dSamples, r, rows);
        if (e == cudaSuccess)
            e = launch_convert_storage(h->dSamples, h->dSamples16 + (size_t)r * pitch,
                                       h->dScale + r, rows, h->S, h->stride, h->storage, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// error message of a handle-less call, read back with hpss_last_error(NULL)
void set_thread_error(const std::string &msg) { g_createError = msg; }
}  // namespace hpss

extern "C" {

const char *hpss_version(void) { return kVersion; }

hpss_status hpss_device_count(int *count) {
    if (!count) return HPSS_ERR_INVALID_ARGUMENT;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        *count = 0;
        return set_error(nullptr, HPSS_ERR_NO_DEVICE,
                         std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
    }
    *count = n;
    return HPSS_OK;
}

hpss_status hpss_create(int device, hpss_handle *out) {
    if (!out) return set_error(nullptr, HPSS_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return set_error(nullptr, HPSS_ERR_NO_DEVICE,
                         "No CUDA devices found on your system.");
    if (device < 0 || device >= n)
        return set_error(nullptr, HPSS_ERR_INVALID_ARGUMENT, "device index out of range");
    hpss_handle h = new (std::nothrow) hpss_handle_s();
    if (!h) return set_error(nullptr, HPSS_ERR_OUT_OF_MEMORY, "host allocation failed");
    h->device = device;
    e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev1);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev2);
    if (e != cudaSuccess) {
        std::string msg = std::string("device init failed: ") + cudaGetErrorString(e);
        hpss_destroy(h);
        return set_error(nullptr, HPSS_ERR_CUDA, msg);
    }
    *out = h;
    return HPSS_OK;
}

hpss_status hpss_destroy(hpss_handle h) {
    if (!h) return HPSS_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_gather(h);
    for (auto *b : {&h->params, &h->chunkBounds, &h->selFirst, &h->selCount, &h->selIdx,
                    &h->candFirst, &h->candCount, &h->notUsed, &h->errWord, &h->m0s,
                    &h->out, &h->octCands, &h->prior, &h->partial, &h->octTab, &h->order,
                    &h->octH0sDev, &h->m0v, &h->deBoxes})
        release(h, *b);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->ev2) cudaEventDestroy(h->ev2);
    if (h->copyStream) {
        cudaStreamSynchronize(h->copyStream);
        cudaStreamDestroy(h->copyStream);
    }
    for (cudaEvent_t e : h->streamEvents) cudaEventDestroy(e);
    if (h->streamT0) cudaEventDestroy(h->streamT0);
    if (h->streamT1) cudaEventDestroy(h->streamT1);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return HPSS_OK;
}

const char *hpss_last_error(hpss_handle h) {
    return h ? h->lastError.c_str() : g_createError.c_str();
}

hpss_status hpss_upload_gather(hpss_handle h, const float *samples,
                               const float *midpoints, const float *halfoffsets,
                               uint32_t nTraces, uint32_t samplesPerTrace,
                               float dtInSeconds, int storage) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    hpss_status rc = prepare_line(h, samples, midpoints, halfoffsets, nTraces, samplesPerTrace,
                                  dtInSeconds, storage);
    if (rc != HPSS_OK) return rc;
    if (nTraces && h->stride != h->S && storage == HPSS_STORAGE_FP32)
        HPSS_CUDA_TRY(h, cudaMemsetAsync(h->dSamples, 0,
                                         (size_t)nTraces * h->stride * sizeof(float), h->stream));
    HPSS_CUDA_TRY(h, copy_line_rows(h, samples, 0, nTraces, h->stream));
    HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    release_upload_staging(h);
    h->gatherReady = true;
    return HPSS_OK;
}

hpss_status hpss_set_traveltime(hpss_handle h, int model, uint32_t nParams,
                                const float *lower, const float *upper, float apm,
                                float h0) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (model < HPSS_MODEL_CMP || model > HPSS_MODEL_OCT)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "Invalid traveltime model");
    if ((int)nParams != model_params(model) || !lower || !upper)
        return set_error(h, HPSS_ERR_LOGIC,
                         "model requires exact " + std::to_string(model_params(model)) +
                             " lower and upper bounds.");
    for (uint32_t j = 0; j < nParams; j++)
        if (!std::isfinite(lower[j]) || !std::isfinite(upper[j]))
            return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "bounds must be finite");
    // the first parameter is a velocity, stored as 4/v^2
    if (!(lower[0] > 0.f) || !(upper[0] > 0.f) || !std::isfinite(4.f / (lower[0] * lower[0])) ||
        !std::isfinite(4.f / (upper[0] * upper[0])))
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "velocity bounds must be > 0");
    h->model = model;
    h->np = nParams;
    for (uint32_t j = 0; j < 3; j++) {
        h->lower[j] = j < nParams ? lower[j] : 0.f;
        h->upper[j] = j < nParams ? upper[j] : 0.f;
    }
    h->apm = apm;
    h->h0 = model == HPSS_MODEL_OCT ? h0 : 0.f;
    h->octCandsHost.clear();
    return HPSS_OK;
}

hpss_status hpss_set_precision(hpss_handle h, int flags) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (flags & ~(HPSS_PREC_FP64_TRAVELTIME | HPSS_PREC_COMPENSATED | HPSS_PREC_FP64))
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "unknown precision flags");
    h->precisionMode = (flags & HPSS_PREC_FP64_TRAVELTIME ? kPrecTt64 : 0) |
                       (flags & HPSS_PREC_COMPENSATED ? kPrecCompensated : 0) |
                       (flags & HPSS_PREC_FP64 ? kPrecF64 : 0);
    return HPSS_OK;
}

hpss_status hpss_set_oct_half_offsets(hpss_handle h, const float *h0s, uint32_t nH0) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (nH0 > kMaxOctHalfOffsets)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT,
                         "at most " + std::to_string(kMaxOctHalfOffsets) + " half-offsets");
    if (nH0 && !h0s) return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "null half-offset array");
    for (uint32_t b = 0; b < nH0; b++)
        if (!std::isfinite(h0s[b]))
            return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "half-offsets must be finite");
    cudaSetDevice(h->device);
    // earlier calls may still read the device copy
    HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (nH0) {
        HPSS_CUDA_TRY(h, ensure(h, h->octH0sDev, nH0 * sizeof(float)));
        HPSS_CUDA_TRY(h, cudaMemcpy(h->octH0sDev.p, h0s, nH0 * sizeof(float),
                                    cudaMemcpyHostToDevice));
    }
    h->octH0s.assign(h0s, h0s + nH0);
    return HPSS_OK;
}

hpss_status hpss_set_grid_mode(hpss_handle h, int mode) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (mode != HPSS_GRID_REFERENCE && mode != HPSS_GRID_INCLUSIVE)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "unknown grid mode");
    h->gridMode = mode;
    return HPSS_OK;
}

hpss_status hpss_set_window(hpss_handle h, int tauIndexDisplacement) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (tauIndexDisplacement < 0 || 2 * tauIndexDisplacement + 1 > kMaxWindow)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT,
                         "window 2*tau+1 must be in [1, 31] (MAX_WINDOW_SIZE)");
    h->tau = tauIndexDisplacement;
    return HPSS_OK;
}

hpss_status hpss_linear_search_device(hpss_handle h, const float *d_m0s, uint32_t nM0,
                                      const uint32_t *granularity, int kernel,
                                      float *d_out, hpss_stats *stats) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (nM0 && (!d_m0s || !d_out))
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "null device pointer");
    return linear_search_impl(h, d_m0s, nM0, granularity, kernel, d_out, stats, false);
}

hpss_status hpss_linear_search(hpss_handle h, const float *m0s, uint32_t nM0,
                               const uint32_t *granularity, int kernel, float *out,
                               hpss_stats *stats) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (nM0 && (!m0s || !out))
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "null host pointer");
    hpss_status rc = check_ready(h);
    if (rc != HPSS_OK) return rc;
    if (nM0 == 0) return HPSS_OK;
    cudaSetDevice(h->device);
    const size_t outElems = (size_t)nM0 * h0_blocks(h) * (2 + h->np) * h->S;
    HPSS_CUDA_TRY(h, ensure(h, h->m0s, nM0 * sizeof(float)));
    HPSS_CUDA_TRY(h, ensure(h, h->out, outElems * sizeof(float)));
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(h->m0s.p, m0s, nM0 * sizeof(float),
                                     cudaMemcpyHostToDevice, h->stream));
    rc = linear_search_impl(h, static_cast<float *>(h->m0s.p), nM0, granularity, kernel,
                            static_cast<float *>(h->out.p), stats, true);
    if (rc != HPSS_OK) return rc;
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(out, h->out.p, outElems * sizeof(float),
                                     cudaMemcpyDeviceToHost, h->stream));
    HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return HPSS_OK;
}

hpss_status hpss_linear_search_line(hpss_handle h, const float *samples,
                                    const float *midpoints, const float *halfoffsets,
                                    uint32_t nTraces, uint32_t samplesPerTrace,
                                    float dtInSeconds, int storage, const float *m0s,
                                    uint32_t nM0, const uint32_t *granularity, int kernel,
                                    float *out, hpss_stats *stats) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (nM0 && (!m0s || !out))
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "null host pointer");
    if (h->model < 0 || h->tau < 0)
        return set_error(h, HPSS_ERR_NOT_READY,
                         "traveltime and window must be set before the line");
    if (!granularity) return set_error(h, HPSS_ERR_LOGIC, "granularity is required");
    if (h0_blocks(h) > 1)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT,
                         "several OCT half-offsets: upload the line and call "
                         "hpss_linear_search instead");
    hpss_status rc = prepare_line(h, samples, midpoints, halfoffsets, nTraces, samplesPerTrace,
                                  dtInSeconds, storage);
    if (rc != HPSS_OK) return rc;
    rc = stream_line_and_search(h, samples, m0s, nM0, granularity, kernel, out, stats);
    if (rc != HPSS_OK) {
        // leave no half-copied line behind
        cudaStreamSynchronize(h->copyStream);
        cudaStreamSynchronize(h->stream);
        h->gatherReady = false;
    }
    return rc;
}

hpss_status hpss_select_traces(hpss_handle h, const float *m0s, uint32_t nM0,
                               uint32_t *counts) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (nM0 && (!m0s || !counts))
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "null host pointer");
    if (!h->gatherReady || h->model < 0)
        return set_error(h, HPSS_ERR_NOT_READY, "gather and traveltime must be set");
    if (nM0 == 0) return HPSS_OK;
    cudaSetDevice(h->device);
    HPSS_CUDA_TRY(h, ensure(h, h->m0s, nM0 * sizeof(float)));
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(h->m0s.p, m0s, nM0 * sizeof(float),
                                     cudaMemcpyHostToDevice, h->stream));
    LsParams lp;
    fill_line_params(h, lp);
    lp.m0s = static_cast<float *>(h->m0s.p);
    lp.nM0 = nM0;
    HPSS_CUDA_TRY(h, expand_h0_blocks(h, lp));  // counts [nH0][nM0] for an h0 list
    hpss_status rc = run_selection(h, lp.m0s, lp.nM0, lp);
    if (rc != HPSS_OK) return rc;
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(counts, lp.selCount, lp.nM0 * sizeof(uint32_t),
                                     cudaMemcpyDeviceToHost, h->stream));
    HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return HPSS_OK;
}

hpss_status hpss_differential_evolution_device(hpss_handle h, const float *d_m0s,
                                               uint32_t nM0, uint32_t population,
                                               uint32_t generations, float F, float CR,
                                               uint64_t seed, float *d_out, hpss_stats *stats) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    return de_impl(h, d_m0s, nM0, population, generations, F, CR, seed, d_out, stats, false);
}

hpss_status hpss_differential_evolution(hpss_handle h, const float *m0s, uint32_t nM0,
                                        uint32_t population, uint32_t generations, float F,
                                        float CR, uint64_t seed, float *out,
                                        hpss_stats *stats) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    if (nM0 && (!m0s || !out))
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "null host pointer");
    hpss_status rc = check_ready(h);
    if (rc != HPSS_OK) return rc;
    if (nM0 == 0) return HPSS_OK;
    cudaSetDevice(h->device);
    const size_t outElems = (size_t)nM0 * h0_blocks(h) * (2 + h->np) * h->S;
    HPSS_CUDA_TRY(h, ensure(h, h->m0s, nM0 * sizeof(float)));
    HPSS_CUDA_TRY(h, ensure(h, h->out, outElems * sizeof(float)));
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(h->m0s.p, m0s, nM0 * sizeof(float),
                                     cudaMemcpyHostToDevice, h->stream));
    rc = de_impl(h, static_cast<float *>(h->m0s.p), nM0, population, generations, F, CR, seed,
                 static_cast<float *>(h->out.p), stats, true);
    if (rc != HPSS_OK) return rc;
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(out, h->out.p, outElems * sizeof(float),
                                     cudaMemcpyDeviceToHost, h->stream));
    HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return HPSS_OK;
}

hpss_status hpss_stretch_free(hpss_handle h, const float *m0s, uint32_t nM0,
                              const float *params, int nmax, float *out, hpss_stats *stats) {
    if (!h) return HPSS_ERR_INVALID_ARGUMENT;
    hpss_status rc = check_ready(h);
    if (rc != HPSS_OK) return rc;
    if (nmax < 0 || nmax > 4096)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "nmax must be in [0, 4096]");
    if (nM0 == 0) return HPSS_OK;
    if (!m0s || !params || !out)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "null host pointer");
    cudaSetDevice(h->device);
    const size_t priorElems = (size_t)nM0 * h0_blocks(h) * h->np * h->S;
    const size_t outElems = (size_t)nM0 * h0_blocks(h) * 3 * h->S;
    HPSS_CUDA_TRY(h, ensure(h, h->m0s, nM0 * sizeof(float)));
    HPSS_CUDA_TRY(h, ensure(h, h->out, outElems * sizeof(float)));
    HPSS_CUDA_TRY(h, ensure(h, h->prior, priorElems * sizeof(float)));
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(h->m0s.p, m0s, nM0 * sizeof(float),
                                     cudaMemcpyHostToDevice, h->stream));
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(h->prior.p, params, priorElems * sizeof(float),
                                     cudaMemcpyHostToDevice, h->stream));
    LsParams lp;
    fill_line_params(h, lp);
    lp.m0s = static_cast<float *>(h->m0s.p);
    lp.nM0 = nM0;
    // several OCT half-offsets: nH0 blocks of the midpoints, one launch
    HPSS_CUDA_TRY(h, use_oct_table(h, lp));
    HPSS_CUDA_TRY(h, expand_h0_blocks(h, lp));
    const float *d_m0s = lp.m0s;
    nM0 = lp.nM0;
    lp.out = static_cast<float *>(h->out.p);
    lp.prior = static_cast<float *>(h->prior.p);
    lp.nmax = nmax;
    HPSS_CUDA_TRY(h, ensure(h, h->notUsed, nM0 * sizeof(unsigned long long)));
    lp.notUsed = static_cast<unsigned long long *>(h->notUsed.p);
    HPSS_CUDA_TRY(h, cudaMemsetAsync(lp.notUsed, 0, nM0 * sizeof(unsigned long long), h->stream));
    HPSS_CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream));
    HPSS_CUDA_TRY(h, ensure(h, h->selFirst, nM0 * sizeof(uint32_t)));
    HPSS_CUDA_TRY(h, ensure(h, h->selCount, nM0 * sizeof(uint32_t)));
    lp.selFirst = static_cast<uint32_t *>(h->selFirst.p);
    lp.selCount = static_cast<uint32_t *>(h->selCount.p);
    lp.selIdx = nullptr;
    if (h->model != HPSS_MODEL_OCT) {
        HPSS_CUDA_TRY(h, launch_select_range(h->dMid, h->nTraces, d_m0s, nM0,
                                             h->model == HPSS_MODEL_CMP ? 0 : 1, h->apm, 0.f,
                                             static_cast<uint32_t *>(h->selFirst.p),
                                             static_cast<uint32_t *>(h->selCount.p), h->stream));
    } else {
        uint64_t total = 0;
        rc = oct_candidate_slots(h, d_m0s, nM0, static_cast<uint32_t *>(h->selFirst.p), &total);
        if (rc != HPSS_OK) return rc;
        const uint32_t *cf = static_cast<const uint32_t *>(h->candFirst.p);
        const uint32_t *cc = static_cast<const uint32_t *>(h->candCount.p);
        lp.selIdx = static_cast<uint32_t *>(h->selIdx.p);
        HPSS_CUDA_TRY(h, launch_sf_select_oct(lp, cf, cc, static_cast<uint32_t *>(h->selIdx.p),
                                              static_cast<uint32_t *>(h->selCount.p), total,
                                              h->stream));
    }
    HPSS_CUDA_TRY(h, cudaEventRecord(h->ev1, h->stream));
    const uint64_t units = (uint64_t)nM0 * h->S;
    if (units > 0xffffffffull)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "too many (midpoint, sample) units");
    // the precision mode with every step in FP64 applies to stretch-free too
    HPSS_CUDA_TRY(h, (h->precisionMode & kPrecF64)
                         ? launch_sf_f64(lp, h->model, (uint32_t)units, h->stream)
                         : launch_sf(lp, h->model, num_sms(h), h->stream));
    HPSS_CUDA_TRY(h, cudaEventRecord(h->ev2, h->stream));
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(out, lp.out, outElems * sizeof(float),
                                     cudaMemcpyDeviceToHost, h->stream));
    HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        std::vector<uint32_t> cnt(nM0);
        std::vector<unsigned long long> nu(nM0);
        HPSS_CUDA_TRY(h, cudaMemcpy(cnt.data(), lp.selCount, nM0 * sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost));
        HPSS_CUDA_TRY(h, cudaMemcpy(nu.data(), lp.notUsed, nM0 * sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost));
        double sel = 0, nus = 0;
        for (uint32_t i = 0; i < nM0; i++) {
            sel += cnt[i];
            nus += (double)nu[i];
        }
        stats->selected_traces = sel;
        stats->evals = sel * (double)h->S * (double)(2 * nmax + 1);
        stats->not_used = nus;
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev1, h->ev2);
        stats->kernel_ms = ms;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        stats->selection_ms = ms;
        stats->kernel_variant = -1;
    }
    return HPSS_OK;
}

void *hpss_stream(hpss_handle h) { return h ? static_cast<void *>(h->stream) : nullptr; }

size_t hpss_device_bytes(hpss_handle h) { return h ? h->deviceBytes : 0; }

}  // extern "C"
