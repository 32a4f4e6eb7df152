// hpss_internal.h -- internal declarations shared by the host and device
// translation units of libhpss_gb300.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

namespace hpss {

constexpr int kModelCmp = 0;
constexpr int kModelZocrs = 1;
constexpr int kModelOct = 2;

// MAX_WINDOW_SIZE (common/include/gpu/interface.h:10) is 32; odd windows up
// to 31 are accepted.
constexpr int kMaxWindow = 31;

// Tuned kernel geometry: a CTA owns 32 consecutive t0 samples (one per lane)
// of one midpoint, its 8 warps split the candidates.
constexpr int kTileSamples = 32;
constexpr int kTunedWarps = 8;
constexpr int kTunedThreads = kTileSamples * kTunedWarps;
constexpr int kPlainThreads = 128;

// Candidate grid modes (HPSS_GRID_* of hpss.h).
constexpr int kGridReference = 0;
constexpr int kGridInclusive = 1;

// Precision modes of the linear search (HPSS_PREC_* of hpss.h).
constexpr int kPrecTt64 = 1;
constexpr int kPrecCompensated = 2;
constexpr int kPrecF64 = 4;  // every step in FP64 (ls_f64.cu)

// Near-tie tolerance (HPSS_NEAR_TIE_REL of hpss.h).
constexpr float kNearTieRel = 1e-4f;

// Device error word bits.
constexpr uint32_t kErrSmemBounds = 1u << 0;
constexpr uint32_t kErrSpanOverflow = 1u << 1;
constexpr uint32_t kErrTimeout = 1u << 2;

// Everything a linear-search (or stretch-free) launch reads and writes.
// Best / runner-up of one candidate range for one (midpoint, sample).
struct PartBest {
    float best, second, stack;
    uint32_t p;
};

struct LsParams {
    // whole line, resident
    const float *samples;     // [nTraces][stride] FP32 (when storage = FP32)
    const uint16_t *samples16;// [nTraces][stride] BF16/FP16
    const float *scale;       // [nTraces] FP16 per-trace scale
    int storage;              // HPSS_STORAGE_* of samples16 (tuned kernel staging)
    uint32_t stride;          // samples per row in memory (>= S, mult. of 8)
    uint32_t S;
    float dt;
    int tau;
    int w;
    const float *mid;
    const float *hoff;
    const float *hsq;         // h*h in float, as copyOnlySelectedTracesToDevice
    // per-midpoint selection
    const float *m0s;
    uint32_t nM0;
    const uint32_t *selFirst; // [nM0]
    const uint32_t *selCount; // [nM0]
    const uint32_t *selIdx;   // nullptr: trace = first + q; else selIdx[first + q]
    // candidates (reference parameter array layout, AoS [P][np])
    const float *params;
    uint32_t P;
    int np;
    // per-chunk parameter bounds for the tuned kernel: [nChunks][2*np]
    const float *chunkBounds;
    uint32_t chunkSize;
    uint32_t nChunks;
    float apm;
    float h0;
    // outputs
    float *out;               // [nM0][2+np][S]
    unsigned long long *notUsed; // [nM0] (may be null)
    unsigned long long *nearTies = nullptr; // one counter (may be null)
    uint32_t *errorWord;
    // stretch-free: prior parameters [nM0][np][S] (raw), n range
    const float *prior;
    int nmax;
    // candidate split of the tuned pair kernel: the chunks are cut into
    // `parts` contiguous ranges of chunksPerPart chunks; with parts > 1 every
    // (midpoint, tile, part) unit writes its range's best / runner-up to
    // `partial` ([nM0][parts][S]) and launch_merge_parts writes the result
    // block.  parts = 1: one unit per (midpoint, tile), written directly.
    uint32_t parts = 1;
    uint32_t chunksPerPart = 0;
    PartBest *partial = nullptr;
    // work queue of the tuned pair kernel: units are taken from
    // *unitCounter (zeroed before the launch; nullptr: static round-robin)
    // and mapped to midpoints through `order` (heaviest first; nullptr:
    // identity)
    uint32_t *unitCounter = nullptr;
    const uint32_t *order = nullptr;
    // OCT: per-trace factors {m, gamma^2, 16 h^2 h0^2, h^2 - h0^2} for the
    // line's h0 (launch_oct_trace_table); read by the OCT tuned and DE kernels
    const float4 *octTab = nullptr;
    // OCT with h0 = 0: warps drop traces by the displaced-midpoint box test
    // (oct_box_may_pass) before the per-sample test
    bool octBox = false;
    // OCT over several target half-offsets in one launch: the launch's nM0
    // midpoints are blocks of m0PerH0 midpoints, block b taking half-offset
    // h0s[b] and the factor table octTab + b * octTabStride (oct_line).
    // m0PerH0 = 0: one half-offset, h0 and octTab.
    uint32_t m0PerH0 = 0;
    const float *h0s = nullptr;
    size_t octTabStride = 0;
#ifdef HPSS_CHECKED
    // checked builds only: bytes armed on the tuned kernel's staging barrier
    // beyond what its copies deliver, so that the bounded wait runs out and
    // the kernel reports kErrTimeout (a drill of the timeout path; 0 = off)
    uint32_t stageDrillBytes = 0;
#endif
};

// Checked builds: the staging-timeout drill from the environment variable
// HPSS_STAGE_DRILL (extra bytes, rounded down to 16); no-op otherwise.
inline void set_stage_drill(LsParams &p) {
#ifdef HPSS_CHECKED
    const char *v = std::getenv("HPSS_STAGE_DRILL");
    p.stageDrillBytes = v ? (uint32_t)(std::strtoul(v, nullptr, 10) & 0xfff0ul) : 0u;
#else
    (void)p;
#endif
}

// Differential evolution launch (de.cu).
struct DeParams {
    LsParams ls;          // line, window, selection, outputs
    uint32_t pop;
    uint32_t gens;
    float F, CR;
    uint32_t seedLo, seedHi;
    float lo[3], hi[3];
    uint32_t staged;      // CMP / ZO-CRS: windows read from spans staged in shared memory
};
constexpr uint32_t kDeMaxPopulation = 128;
// Target half-offsets of one OCT call (hpss_set_oct_half_offsets).
constexpr uint32_t kMaxOctHalfOffsets = 64;

struct Handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    std::string lastError;
    // line
    uint32_t nTraces = 0, S = 0, stride = 0;
    float dt = 0;
    int storage = 0;
    bool gatherReady = false;
    float *dSamples = nullptr;
    uint16_t *dSamples16 = nullptr;
    float *dScale = nullptr;
    float *dMid = nullptr, *dHoff = nullptr, *dHsq = nullptr;
    // the per-trace arrays (mid, hoff, hsq, scale) are slices of dTraceBuf;
    // allocated bytes of the line buffers, kept across uploads that fit
    void *dTraceBuf = nullptr;
    size_t capSamples = 0, capSamples16 = 0, capTrace = 0;
    std::vector<float> hMid, hHoff, hHsq;
    // second stream and events of the streamed line upload
    // (hpss_linear_search_line): amplitude chunks arrive on copyStream
    cudaStream_t copyStream = nullptr;
    std::vector<cudaEvent_t> streamEvents;
    cudaEvent_t streamT0 = nullptr, streamT1 = nullptr;  // timed span of a streamed call
    // traveltime
    int model = -1;
    uint32_t np = 0;
    float lower[3] = {0, 0, 0}, upper[3] = {0, 0, 0};
    float apm = 0, h0 = 0;
    int tau = -1;
    int gridMode = kGridReference;
    int precisionMode = 0;
    // scratch (grown on demand, owned by the handle)
    void *scratch = nullptr;
    size_t scratchBytes = 0;
    void *pinned = nullptr;
    size_t pinnedBytes = 0;
    size_t deviceBytes = 0;
};

// Launchers (ls_kernels.cu).
cudaError_t launch_build_grid(int model, int mode, const float *lower, const float *inc,
                              const float *last, const uint32_t *gran, float *params,
                              uint32_t P, cudaStream_t st);
cudaError_t launch_chunk_bounds(const LsParams &p, float *bounds,
                                cudaStream_t st);
// precisionMode: kPrecTt64 | kPrecCompensated (0: the reference's FP32 arithmetic)
cudaError_t launch_ls_plain(const LsParams &p, cudaStream_t st, int precisionMode = 0);
// The linear search and the stretch-free stack with every step in FP64
// (kPrecF64, ls_f64.cu); nUnits = nM0 * S.
cudaError_t launch_ls_f64(const LsParams &p, cudaStream_t st);
cudaError_t launch_sf_f64(const LsParams &p, int model, uint32_t nUnits, cudaStream_t st);
// Tuned pair kernel (CMP / ZO-CRS) shapes, `variant`: 0 = 2 candidate pairs
// per thread, 2 CTAs/SM; 1 = 1 pair, 3 CTAs/SM; 2 = 2 pairs, 3 CTAs/SM
// (chunk = 8 warps x 2*pairs candidates).  exactStack selects the
// instantiations that accumulate the stack's linear sum in the reference's
// order.
cudaError_t launch_ls_tuned_cmp(const LsParams &p, uint32_t grid, uint32_t tiles,
                                uint32_t nUnits, cudaStream_t st, int variant,
                                bool exactStack);
cudaError_t launch_ls_tuned_zocrs(const LsParams &p, uint32_t grid, uint32_t tiles,
                                  uint32_t nUnits, cudaStream_t st, int variant,
                                  bool exactStack);
// 16-bit rows staged by bulk copies (S16 instantiations)
cudaError_t launch_ls_tuned_cmp16(const LsParams &p, uint32_t grid, uint32_t tiles,
                                  uint32_t nUnits, cudaStream_t st, int variant);
cudaError_t launch_ls_tuned_zocrs16(const LsParams &p, uint32_t grid, uint32_t tiles,
                                    uint32_t nUnits, cudaStream_t st, int variant);
cudaError_t launch_ls_tuned_cmp_exact(const LsParams &p, uint32_t grid, uint32_t tiles,
                                      uint32_t nUnits, cudaStream_t st, int variant);
cudaError_t launch_ls_tuned_zocrs_exact(const LsParams &p, uint32_t grid, uint32_t tiles,
                                        uint32_t nUnits, cudaStream_t st, int variant);
// Tuned kernel for OCT (ls_oct.cu): (midpoint, 32-sample tile, candidate
// part) units, windows read through L1, parts merged in candidate order.
// `partial` holds oct_partial_bytes(nM0, S, parts) bytes.
uint32_t oct_parts(const LsParams &p, uint32_t numSms);
size_t oct_partial_bytes(uint32_t nM0, uint32_t S, uint32_t parts);
// tt64: the displaced midpoint and time in FP64 (HPSS_PREC_FP64_TRAVELTIME).
cudaError_t launch_ls_oct(const LsParams &p, uint32_t numSms, void *partial, uint32_t parts,
                          cudaStream_t st, bool tt64 = false);
// Tuned pair kernel with a precision mode (prec: kPrecTt64 | kPrecCompensated,
// not 0), shape 1 (one candidate pair per thread, 3 CTAs/SM; chunk of 16),
// linear sum from the per-tap sums (ls_tuned_prec.cu).
cudaError_t launch_ls_tuned_prec(const LsParams &p, int model, int prec, uint32_t grid,
                                 uint32_t tiles, uint32_t nUnits, cudaStream_t st);
// Per-trace factors of the OCT formulas for half-offset h0 (ls_oct.cu).
cudaError_t launch_oct_trace_table(const float *mid, const float *hoff, uint32_t n, float h0,
                                   float4 *tab, cudaStream_t st);
// order[] = midpoints by descending count[] (select.cu); for up to
// kMaxOrderedMidpoints midpoints per launch.
constexpr uint32_t kMaxOrderedMidpoints = 4096;
cudaError_t launch_order_by_count(const uint32_t *count, uint32_t n, uint32_t *order,
                                  cudaStream_t st);
// Combine `parts` candidate ranges of every (midpoint, sample) in candidate
// order and write the result block [nM0][2+np][S]; counts near-ties.
cudaError_t launch_merge_parts(const LsParams &p, uint32_t parts, const PartBest *partial,
                               cudaStream_t st);
// Order-preserving compaction of 0 / 1 flags in selIdx (slots p.selFirst[mi]
// .. + candCount[mi]) into the selected trace indices candFirst[mi] + q, in
// place; selCount[mi] = their number (ls_common.cu).
cudaError_t launch_select_compact(const LsParams &p, const uint32_t *candFirst,
                                  const uint32_t *candCount, uint32_t *selIdx,
                                  uint32_t *selCount, cudaStream_t st);
// total: sum of candCount (the selIdx slots, p.selFirst their prefix);
// candBox: {min slope, max slope, min c, max c} of the sampled candidates;
// p.octTab: the factor tables.
cudaError_t launch_select_oct(const LsParams &p, const float *cands,
                              uint32_t nCand, uint32_t *selIdx,
                              uint32_t *selCount, const uint32_t *candFirst,
                              const uint32_t *candCount, uint64_t total, float4 candBox,
                              cudaStream_t st);
cudaError_t launch_convert_storage(const float *src, uint16_t *dst,
                                   float *scale, uint32_t nTraces, uint32_t S,
                                   uint32_t stride, int storage,
                                   cudaStream_t st);
cudaError_t launch_de(const DeParams &d, int model, uint32_t numSms, cudaStream_t st);
// stretch-free over p.nM0 midpoints x p.S samples (grid from the SM count)
cudaError_t launch_sf(const LsParams &p, int model, int numSms, cudaStream_t st);
cudaError_t launch_sf_select_oct(const LsParams &p, const uint32_t *candFirst,
                                 const uint32_t *candCount, uint32_t *selIdx,
                                 uint32_t *selCount, uint64_t total, cudaStream_t st);
// boxes: [nM0][S] float4 scratch (the initial populations' slope / c ranges).
cudaError_t launch_de_select_oct(const DeParams &d, const uint32_t *candFirst,
                                 const uint32_t *candCount, uint32_t *selIdx,
                                 uint32_t *selCount, uint64_t total, float4 *boxes,
                                 cudaStream_t st);

}  // namespace hpss
