// hpss_handle.h -- the handle behind the C ABI and the host helpers shared by
// its translation units: hpss_capi.cu (handle, line, setters and the extern
// "C" entry points), ls_host.cu (linear search: autotuner, candidate split,
// work queue, streamed line) and de_host.cu (differential evolution).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/hpss.h"
#include "hpss_internal.h"

struct hpss_handle_s : public hpss::Handle {
    // scratch buffers, grown on demand
    struct Buf {
        void *p = nullptr;
        size_t bytes = 0;
    };
    Buf params, chunkBounds, selFirst, selCount, selIdx, candFirst, candCount,
        notUsed, errWord, m0s, out, octCands, prior, partial, order;
    Buf octTab;                // OCT per-trace factors of the line, one table per
                               // half-offset in octTabH0s
    bool octTabValid = false;
    std::vector<float> octTabH0s;
    // OCT over several target half-offsets (hpss_set_oct_half_offsets):
    // empty = the single h0 of hpss_set_traveltime
    std::vector<float> octH0s;
    Buf octH0sDev;             // octH0s on the device
    Buf m0v;                   // midpoints of a call repeated per half-offset
    Buf deBoxes;               // OCT DE selection: per-sample initial-population boxes
    std::string gridKey;       // grid held in `params` (empty: none)
    uint32_t boundsChunk = 0;  // chunk size of the bounds in `chunkBounds` (0: none)
    std::vector<float> octCandsHost;
    std::map<std::string, int> variantCache;  // autotuner decisions
    int lastVariant = -1;
    uint32_t lastParts = 1;                    // candidate parts of the last search
    uint32_t meanFold = 0;                     // traces per distinct midpoint
};

#define HPSS_CUDA_TRY(h, expr)                                                 \
    do {                                                                       \
        cudaError_t _e = (expr);                                               \
        if (_e != cudaSuccess) {                                               \
            return set_error(h, _e == cudaErrorMemoryAllocation                \
                                    ? HPSS_ERR_OUT_OF_MEMORY                   \
                                    : HPSS_ERR_CUDA,                           \
                             std::string("CUDA error at ") + __FILE__ + ":" +  \
                                 std::to_string(__LINE__) + " (" #expr "): " + \
                                 cudaGetErrorString(_e));                      \
        }                                                                      \
    } while (0)

namespace hpss {

// Sets the handle's (or, without one, the thread's) last error; returns code.
hpss_status set_error(hpss_handle h, hpss_status code, const std::string &msg);
// Grows a handle buffer to at least `bytes` (contents are not kept).
cudaError_t ensure(hpss_handle h, hpss_handle_s::Buf &b, size_t bytes);
void release(hpss_handle h, hpss_handle_s::Buf &b);
hpss_status check_ready(hpss_handle h);
// OCT: the candidate traces of each midpoint (h->candFirst / candCount), their
// slot offsets in selIdx (`first`) and selIdx sized for them (`total` slots,
// rejected at 2^32 or more).
hpss_status oct_candidate_slots(hpss_handle h, const float *d_m0s, uint32_t nM0,
                                uint32_t *first, uint64_t *total);
// Trace selection of nM0 device midpoints into the handle's buffers (lp's
// selFirst / selCount / selIdx are set).
hpss_status run_selection(hpss_handle h, const float *d_m0s, uint32_t nM0, LsParams &lp);
// The resident line, window and traveltime of the handle as kernel parameters.
void fill_line_params(hpss_handle h, LsParams &lp);
// OCT: the per-trace factor tables of the line for the current h0 or
// half-offset list (built on first use after an upload or a change).
cudaError_t use_oct_table(hpss_handle h, LsParams &lp);
// Result blocks per midpoint of an OCT call: the number of target
// half-offsets of hpss_set_oct_half_offsets (1 without a list or for
// CMP / ZO-CRS).
uint32_t h0_blocks(hpss_handle h);
// OCT with several target half-offsets: lp.m0s / lp.nM0 (nM0 midpoints)
// become nH0 * nM0 midpoints in h0 blocks (block b = the midpoints at h0s[b],
// copied on the device) and lp's block fields are set; otherwise nothing
// changes.
cudaError_t expand_h0_blocks(hpss_handle h, LsParams &lp);
int num_sms(hpss_handle h);
// 16-bit storage: free the FP32 staging area of a finished upload.
void release_upload_staging(hpss_handle h);
// Amplitudes of traces [a, b) of a line being uploaded, on stream st.
cudaError_t copy_line_rows(hpss_handle h, const float *samples, uint32_t a, uint32_t b,
                           cudaStream_t st);

cudaError_t launch_select_range(const float *mid, uint32_t n, const float *m0s,
                                uint32_t nM0, int mode, float apm, float radius,
                                uint32_t *first, uint32_t *count,
                                cudaStream_t st);
cudaError_t launch_exclusive_scan(const uint32_t *count, uint32_t *first,
                                  uint32_t n, cudaStream_t st);
size_t tuned_stage_floats();
size_t tuned_stage_floats_min();

// ls_host.cu.  A call that is one group of a larger call
// (hpss_linear_search_line): the counters were cleared once for the whole
// call and this group's per-midpoint counts start at `m0Offset`.
struct GroupOfCall {
    uint32_t m0Offset;
};
hpss_status linear_search_impl(hpss_handle h, const float *d_m0s, uint32_t nM0,
                               const uint32_t *granularity, int kernel, float *d_out,
                               hpss_stats *stats, bool sync,
                               const GroupOfCall *group = nullptr);
// Body of hpss_linear_search_line after the line's geometry is prepared.
hpss_status stream_line_and_search(hpss_handle h, const float *samples, const float *m0s,
                                   uint32_t nM0, const uint32_t *granularity, int kernel,
                                   float *out, hpss_stats *stats);

// de_host.cu
hpss_status de_impl(hpss_handle h, const float *d_m0s, uint32_t nM0, uint32_t pop,
                    uint32_t gens, float F, float CR, uint64_t seed, float *d_out,
                    hpss_stats *stats, bool sync);

}  // namespace hpss
