// ls_host.cu -- host side of the linear search behind the C ABI: the tuned
// kernel's shapes and autotuner, the candidate split of small calls, the
// work queue, the launch sequence (grid -> selection -> order -> semblance
// kernel, merged parts) and the streamed line upload + search.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "hpss_handle.h"

namespace hpss {

// Shapes of the tuned pair kernel: candidate pairs per thread and resident
// CTAs per SM (more pairs: more independent chains per thread; more CTAs:
// more warps to hide latency, a smaller shared-memory stage).
constexpr int kTunedVariants = 3;
constexpr int kVariantPairs[kTunedVariants] = {2, 1, 2};
constexpr int kVariantCtasPerSm[kTunedVariants] = {2, 3, 3};

// Candidate parts of the pair kernel: a call whose `base` (midpoint, tile)
// units fill fewer than four waves of the resident CTAs is split into
// candidate ranges, at most one per chunk.
uint32_t pair_parts(uint64_t base, uint32_t nChunks, int numSms, int ctasPerSm) {
    const uint64_t want = (uint64_t)numSms * (uint64_t)ctasPerSm * 4;
    if (base == 0 || base >= want) return 1;
    const uint64_t parts = std::min<uint64_t>((want + base - 1) / base, nChunks);
    if (parts <= 1) return 1;
    // equal ranges, none empty
    const uint32_t per = (uint32_t)((nChunks + parts - 1) / parts);
    return (nChunks + per - 1) / per;
}

// Autotuner decisions shared by the handles of the process (keys carry the
// device), so that a handle opened after another one does not tune again.
static std::mutex g_variantMutex;
static std::map<std::string, int> g_variantCache;

// Autotuner: the first time a (device, storage, model, window, candidates,
// samples, fold, candidate split) key is seen, every variant is timed on a
// prefix of the work units (results are overwritten by the real launch) and
// the fastest is cached in the handle and in the process-wide table.
// HPSS_LS_VARIANT=<n> forces a variant.
template <typename SetChunks, typename Launch>
hpss_status choose_variant(hpss_handle h, const LsParams &lp, uint32_t units, bool exactStack,
                           SetChunks setChunks, Launch launch, int *out) {
    if (const char *env = std::getenv("HPSS_LS_VARIANT")) {
        int v = std::atoi(env);
        if (v >= 0 && v < kTunedVariants) {
            *out = v;
            return HPSS_OK;
        }
    }
    // calls split into candidate ranges (few midpoints) have their own entry:
    // the best shape differs from that of a call that fills the GPU by itself
    const uint32_t split =
        pair_parts(units, (lp.P + 2 * kTunedWarps * kVariantPairs[0] - 1) /
                              (2 * kTunedWarps * kVariantPairs[0]),
                   num_sms(h), kVariantCtasPerSm[0]);
    const std::string key = std::to_string(h->device) + "/" + std::to_string(h->storage) + "/" +
                            std::to_string(h->model) + "/" + std::to_string(exactStack) + "/" +
                            std::to_string(lp.w) + "/" +
                            std::to_string(lp.P) + "/" + std::to_string(lp.S) + "/" +
                            std::to_string(h->meanFold) + "/" + std::to_string(split);
    auto it = h->variantCache.find(key);
    if (it != h->variantCache.end()) {
        *out = it->second;
        return HPSS_OK;
    }
    {
        // decided already by another handle of this process on this device
        std::lock_guard<std::mutex> lock(g_variantMutex);
        auto g = g_variantCache.find(key);
        if (g != g_variantCache.end()) {
            h->variantCache[key] = g->second;
            *out = g->second;
            return HPSS_OK;
        }
    }
    // trial prefix: at least three waves of the 2-CTA shape and two of the
    // 3-CTA shapes, grown (doubling, up to the whole call) until the first
    // shape's trial takes kTrialMs, so that the launches' timing noise stays
    // small against the shapes' differences; a ZO-CRS unit of 18081
    // candidates takes ~0.3 s, so there the first prefix is long enough
    constexpr float kTrialMs = 4.f;
    uint32_t sub = std::min<uint32_t>(units, (uint32_t)num_sms(h) * 6);
    struct Events {
        cudaEvent_t a = nullptr, b = nullptr;
        ~Events() {
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } ev;
    HPSS_CUDA_TRY(h, cudaEventCreate(&ev.a));
    HPSS_CUDA_TRY(h, cudaEventCreate(&ev.b));
    cudaEvent_t a = ev.a, b = ev.b;
    auto trial = [&](int v, uint32_t n, float *ms) -> hpss_status {
        HPSS_CUDA_TRY(h, setChunks(2 * kVariantPairs[v]));
        HPSS_CUDA_TRY(h, cudaEventRecord(a, h->stream));
        HPSS_CUDA_TRY(h, launch(v, n));
        HPSS_CUDA_TRY(h, cudaEventRecord(b, h->stream));
        HPSS_CUDA_TRY(h, cudaEventSynchronize(b));
        HPSS_CUDA_TRY(h, cudaEventElapsedTime(ms, a, b));
        return HPSS_OK;
    };
    for (int v = 0; v < kTunedVariants; v++) {  // first-launch costs
        HPSS_CUDA_TRY(h, setChunks(2 * kVariantPairs[v]));
        HPSS_CUDA_TRY(h, launch(v, std::min<uint32_t>(sub, 64)));
    }
    float t0ms = 0;
    hpss_status trc = trial(0, sub, &t0ms);
    if (trc != HPSS_OK) return trc;
    while (t0ms < kTrialMs && sub < units) {
        sub = (uint32_t)std::min<uint64_t>((uint64_t)sub * 2, units);
        trc = trial(0, sub, &t0ms);
        if (trc != HPSS_OK) return trc;
    }
    // every shape timed on the same prefix, twice in alternating order when
    // a trial is short (the faster of the two counts); shape 0 stays unless
    // another is faster by more than the noise margin
    float tms[kTunedVariants];
    tms[0] = t0ms;
    const int rounds = t0ms < 50.f ? 2 : 1;
    for (int r = 0; r < rounds; r++) {
        for (int i = 0; i < kTunedVariants; i++) {
            const int v = r % 2 ? kTunedVariants - 1 - i : i;
            if (r == 0 && v == 0) continue;  // timed above
            float ms = 0;
            trc = trial(v, sub, &ms);
            if (trc != HPSS_OK) return trc;
            tms[v] = r == 0 ? ms : std::min(tms[v], ms);
        }
    }
    int bestV = 0;
    for (int v = 1; v < kTunedVariants; v++)
        if (tms[v] < tms[bestV] * 0.985f) bestV = v;
    h->variantCache[key] = bestV;
    {
        std::lock_guard<std::mutex> lock(g_variantMutex);
        g_variantCache.emplace(key, bestV);
    }
    *out = bestV;
    return HPSS_OK;
}

hpss_status linear_search_impl(hpss_handle h, const float *d_m0s, uint32_t nM0,
                               const uint32_t *granularity, int kernel,
                               float *d_out, hpss_stats *stats, bool sync,
                               const GroupOfCall *group) {
    hpss_status rc = check_ready(h);
    if (rc != HPSS_OK) return rc;
    if (!granularity)
        return set_error(h, HPSS_ERR_LOGIC, "granularity is required");
    if (kernel != HPSS_KERNEL_PLAIN && kernel != HPSS_KERNEL_TUNED &&
        kernel != HPSS_KERNEL_TUNED_EXACT)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "unknown kernel family");
    const bool tuned = kernel != HPSS_KERNEL_PLAIN;
    const bool exactStack = kernel == HPSS_KERNEL_TUNED_EXACT;
    uint64_t P = 1;
    uint32_t gran[3] = {1, 1, 1};
    float inc[3] = {0, 0, 0}, low[3] = {0, 0, 0}, last[3] = {0, 0, 0};
    for (uint32_t j = 0; j < h->np; j++) {
        if (granularity[j] == 0)
            return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "granularity must be > 0");
        gran[j] = granularity[j];
        P *= granularity[j];
        if (h->gridMode == kGridReference) {
            low[j] = h->lower[j];
            // setupDiscretizationSteps (LinearSearchAlgorithm.cpp:137-139)
            inc[j] = (h->upper[j] - h->lower[j]) / static_cast<float>(granularity[j]);
        } else {
            // inclusive: velocity uniform in c = 4/v^2 from c(lower) to c(upper)
            float a = h->lower[j], b = h->upper[j];
            if (j == 0) {
                a = 4.0f / (h->lower[0] * h->lower[0]);
                b = 4.0f / (h->upper[0] * h->upper[0]);
            }
            low[j] = a;
            last[j] = b;
            inc[j] = granularity[j] > 1 ? (b - a) / static_cast<float>(granularity[j] - 1) : 0.f;
        }
    }
    if (P > 0x7fffffffull)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "too many candidates");
    if (nM0 == 0) return HPSS_OK;
    cudaSetDevice(h->device);

    LsParams lp;
    fill_line_params(h, lp);
    lp.m0s = d_m0s;
    lp.nM0 = nM0;
    lp.P = (uint32_t)P;
    lp.out = d_out;
    HPSS_CUDA_TRY(h, use_oct_table(h, lp));
    // OCT over several half-offsets: the midpoints in h0 blocks, one search
    if (!group) {
        HPSS_CUDA_TRY(h, expand_h0_blocks(h, lp));
        d_m0s = lp.m0s;
        nM0 = lp.nM0;
    }

    // The candidate grid (and below the chunk bounds) depend only on the
    // model, the bounds, the granularity and the grid mode: a call that
    // repeats the previous call's grid (one midpoint per call) reuses them
    // from the handle's buffers instead of rebuilding them.
    std::string gridKey = std::to_string(h->model) + "/" + std::to_string(h->gridMode) + "/" +
                          std::to_string(h->np) + "/" + std::to_string(P);
    for (uint32_t j = 0; j < h->np; j++) {
        uint32_t bits[3];
        std::memcpy(&bits[0], &low[j], 4);
        std::memcpy(&bits[1], &inc[j], 4);
        std::memcpy(&bits[2], &last[j], 4);
        for (uint32_t b : bits) gridKey += "/" + std::to_string(b);
        gridKey += "/" + std::to_string(gran[j]);
    }
    if (h->gridKey != gridKey) {
        h->gridKey.clear();
        h->boundsChunk = 0;
        HPSS_CUDA_TRY(h, ensure(h, h->params, P * h->np * sizeof(float)));
        HPSS_CUDA_TRY(h, launch_build_grid(h->model, h->gridMode, low, inc, last, gran,
                                           static_cast<float *>(h->params.p), (uint32_t)P,
                                           h->stream));
        h->gridKey = gridKey;
    }
    lp.params = static_cast<float *>(h->params.p);
    // candidates per thread of the tuned kernel: 2 * pairs (CMP / ZO-CRS),
    // 4 (OCT); HPSS_LS_PAIRS overrides the pair count (1, 2 or 4)
    // Tuned kernel: CMP / ZO-CRS run the branch-free pair kernel in one of
    // kTunedVariants shapes (candidate pairs per thread x CTAs per SM), OCT the
    // branchy kernel (4 candidates per thread).  The chunk bounds depend on
    // the chunk size (8 warps x candidates per thread).
    // Precision modes: CMP / ZO-CRS run the pair kernel's precision
    // instantiations (shape 1, not autotuned); OCT the OCT kernel with the
    // FP64 traveltime; OCT with compensated sums runs the plain kernel.
    // Every step in FP64 (kPrecF64) runs the FP64 kernel whatever is asked.
    const int prec = h->precisionMode;
    const bool f64 = (prec & kPrecF64) != 0;
    const bool pairKernel = tuned && !f64 && h->model != HPSS_MODEL_OCT && lp.w <= 15 &&
                            h->stride + 8 <= (uint32_t)tuned_stage_floats_min();
    const bool octKernel = tuned && !f64 && h->model == HPSS_MODEL_OCT && lp.w <= 15 &&
                           !(prec & kPrecCompensated);
    // chunk bounds (read by the pair kernel only), rebuilt when the chunk size
    // or the grid changed
    auto setChunks = [&](int perThread) -> cudaError_t {
        lp.chunkSize = kTunedWarps * perThread;
        lp.nChunks = (lp.P + lp.chunkSize - 1) / lp.chunkSize;
        if (h->boundsChunk != lp.chunkSize) {
            h->boundsChunk = 0;
            cudaError_t e =
                ensure(h, h->chunkBounds, (size_t)lp.nChunks * 2 * h->np * sizeof(float));
            if (e != cudaSuccess) return e;
            e = launch_chunk_bounds(lp, static_cast<float *>(h->chunkBounds.p), h->stream);
            if (e != cudaSuccess) return e;
            h->boundsChunk = lp.chunkSize;
        }
        lp.chunkBounds = static_cast<float *>(h->chunkBounds.p);
        return cudaSuccess;
    };
    // counters, cleared by one memset: error word at byte 0, the pair
    // kernel's work-queue counter at byte 4, near-tie counter at byte 8, the
    // per-midpoint notUsed counts from byte 16
    if (!group) {
        HPSS_CUDA_TRY(h, ensure(h, h->notUsed, 16 + nM0 * sizeof(unsigned long long)));
        HPSS_CUDA_TRY(h, cudaMemsetAsync(h->notUsed.p, 0, 16 + nM0 * sizeof(unsigned long long),
                                         h->stream));
    }
    char *counters = static_cast<char *>(h->notUsed.p);
    lp.errorWord = reinterpret_cast<uint32_t *>(counters);
    lp.nearTies = reinterpret_cast<unsigned long long *>(counters + 8);
    lp.notUsed = reinterpret_cast<unsigned long long *>(counters + 16) +
                 (group ? group->m0Offset : 0);
    set_stage_drill(lp);

    const uint32_t tiles = (h->S + kTileSamples - 1) / kTileSamples;
    const uint64_t units = (uint64_t)nM0 * tiles;
    uint32_t octParts = 1;
    if (octKernel) {
        if (nM0 > 1 && nM0 <= kMaxOrderedMidpoints)
            HPSS_CUDA_TRY(h, ensure(h, h->order, nM0 * sizeof(uint32_t)));
        // per-part best / runner-up of the OCT kernel
        octParts = oct_parts(lp, (uint32_t)num_sms(h));
        HPSS_CUDA_TRY(h, ensure(h, h->partial, oct_partial_bytes(nM0, h->S, octParts)));
    } else if (pairKernel) {
        // midpoints of the batch by descending selected traces (work-queue order)
        if (nM0 > 1 && nM0 <= kMaxOrderedMidpoints)
            HPSS_CUDA_TRY(h, ensure(h, h->order, nM0 * sizeof(uint32_t)));
        // per-part best / runner-up of a split pair-kernel call, for the
        // largest split of any shape (allocated before the timed region)
        uint32_t maxParts = 1;
        for (int v = 0; v < kTunedVariants; v++) {
            const uint32_t chunk = kTunedWarps * 2 * kVariantPairs[v];
            maxParts = std::max(maxParts, pair_parts(units, (lp.P + chunk - 1) / chunk,
                                                     num_sms(h), kVariantCtasPerSm[v]));
        }
        if (maxParts > 1)
            HPSS_CUDA_TRY(h, ensure(h, h->partial, (size_t)nM0 * maxParts * h->S * sizeof(PartBest)));
    }

    HPSS_CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream));
    rc = run_selection(h, d_m0s, nM0, lp);
    if (rc != HPSS_OK) return rc;
    HPSS_CUDA_TRY(h, cudaEventRecord(h->ev1, h->stream));
    // unit indices (and a work-queue counter past the last unit) stay below 2^31
    if (units > 0x7fffffffull)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "too many (midpoint, tile) units");
    // nBase (midpoint, tile) units, each split into the shape's candidate
    // parts; a split launch of all units is followed by the ordered merge
    uint32_t lastParts = 1;
    // work queue of the pair kernel: heaviest midpoints first, units taken
    // from a counter that every launch starts at zero
    const bool ordered = pairKernel && nM0 > 1 && nM0 <= kMaxOrderedMidpoints;
    if (ordered) {
        HPSS_CUDA_TRY(h, launch_order_by_count(lp.selCount, nM0,
                                               static_cast<uint32_t *>(h->order.p), h->stream));
        lp.order = static_cast<const uint32_t *>(h->order.p);
    }
    uint32_t *unitCounter = reinterpret_cast<uint32_t *>(static_cast<char *>(h->notUsed.p) + 4);
    auto launchPair = [&](int variant, uint32_t nBase) -> cudaError_t {
        LsParams q = lp;
        q.parts = pair_parts(units, lp.nChunks, num_sms(h), kVariantCtasPerSm[variant]);
        q.chunksPerPart = (lp.nChunks + q.parts - 1) / q.parts;
        q.partial = static_cast<PartBest *>(h->partial.p);
        lastParts = q.parts;
        const uint64_t nUnits = (uint64_t)nBase * q.parts;
        if (nUnits > 0x7fffffffull) return cudaErrorInvalidConfiguration;
        const uint32_t grid = (uint32_t)std::min<uint64_t>(
            nUnits, (uint64_t)num_sms(h) * kVariantCtasPerSm[variant]);
        // more units than resident CTAs: take them from the work queue
        if (nUnits > grid) {
            q.unitCounter = unitCounter;
            cudaError_t e0 = cudaMemsetAsync(unitCounter, 0, sizeof(uint32_t), h->stream);
            if (e0 != cudaSuccess) return e0;
        }
        cudaError_t e =
            prec ? launch_ls_tuned_prec(q, h->model, prec, grid, tiles, (uint32_t)nUnits,
                                        h->stream)
            : h->model == HPSS_MODEL_CMP
                ? launch_ls_tuned_cmp(q, grid, tiles, (uint32_t)nUnits, h->stream, variant,
                                      exactStack)
                : launch_ls_tuned_zocrs(q, grid, tiles, (uint32_t)nUnits, h->stream, variant,
                                        exactStack);
        if (e != cudaSuccess || q.parts == 1 || nBase != units) return e;
        return launch_merge_parts(q, q.parts, q.partial, h->stream);
    };
    int variant = 0;
    if (pairKernel && prec) {
        variant = 1;  // the precision instantiations' shape
        HPSS_CUDA_TRY(h, setChunks(2 * kVariantPairs[variant]));
    } else if (pairKernel) {
        // the autotuner's timing launches (a prefix of the units) count no
        // near-ties
        unsigned long long *ties = lp.nearTies;
        lp.nearTies = nullptr;
        rc = choose_variant(h, lp, (uint32_t)units, exactStack, setChunks, launchPair, &variant);
        lp.nearTies = ties;
        if (rc != HPSS_OK) return rc;
        HPSS_CUDA_TRY(h, setChunks(2 * kVariantPairs[variant]));
        HPSS_CUDA_TRY(h, cudaEventRecord(h->ev1, h->stream));
    }
    if (pairKernel) {
        HPSS_CUDA_TRY(h, launchPair(variant, (uint32_t)units));
    } else if (octKernel) {
        // work queue as for the pair kernel
        if (nM0 > 1 && nM0 <= kMaxOrderedMidpoints) {
            HPSS_CUDA_TRY(h, launch_order_by_count(lp.selCount, nM0,
                                                   static_cast<uint32_t *>(h->order.p),
                                                   h->stream));
            lp.order = static_cast<const uint32_t *>(h->order.p);
        }
        lp.unitCounter = unitCounter;
        HPSS_CUDA_TRY(h, cudaMemsetAsync(unitCounter, 0, sizeof(uint32_t), h->stream));
        HPSS_CUDA_TRY(h, launch_ls_oct(lp, (uint32_t)num_sms(h), h->partial.p, octParts,
                                       h->stream, (prec & kPrecTt64) != 0));
    } else {
        HPSS_CUDA_TRY(h, f64 ? launch_ls_f64(lp, h->stream)
                             : launch_ls_plain(lp, h->stream, h->precisionMode));
    }
    h->lastVariant = pairKernel ? variant : -1;
    h->lastParts = pairKernel ? lastParts : octKernel ? octParts : 1;
    HPSS_CUDA_TRY(h, cudaEventRecord(h->ev2, h->stream));

    if (stats || sync) {
        HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        uint32_t err = 0;
        unsigned long long ties = 0;
        HPSS_CUDA_TRY(h, cudaMemcpy(&err, lp.errorWord, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        HPSS_CUDA_TRY(h, cudaMemcpy(&ties, lp.nearTies, sizeof(ties), cudaMemcpyDeviceToHost));
        if (stats) {
            std::memset(stats, 0, sizeof(*stats));
            stats->near_ties = (double)ties;
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
            stats->evals = sel * (double)h->S * (double)P;
            stats->not_used = nus;
            float ms = 0;
            cudaEventElapsedTime(&ms, h->ev1, h->ev2);
            stats->kernel_ms = ms;
            cudaEventElapsedTime(&ms, h->ev0, h->ev1);
            stats->selection_ms = ms;
            stats->device_error = err;
            stats->kernel_variant = h->lastVariant;
            stats->candidate_parts = h->lastParts;
        }
        if (err & kErrTimeout)
            return set_error(h, HPSS_ERR_TIMEOUT,
                             "staging copies did not complete in time, error word " +
                                 std::to_string(err));
        if (err)
            return set_error(h, HPSS_ERR_DEVICE_CHECK,
                             "device check failed, error word " + std::to_string(err));
    }
    return HPSS_OK;
}

// Body of hpss_linear_search_line, after prepare_line: the amplitudes go
// to the device in trace ranges on the copy stream, the midpoints are
// searched in contiguous groups on the handle's
// stream, each group waiting only for the chunk that holds the last trace
// its midpoints can select, and each group's results go back on the copy
// stream while the next group runs.  HPSS_STREAM_CHUNKS / HPSS_STREAM_GROUPS
// (1 .. 64) set the numbers of trace ranges and midpoint groups.
constexpr uint32_t kStreamChunks = 8, kStreamGroups = 8, kStreamMax = 64;

static uint32_t stream_count(const char *name, uint32_t dflt) {
    const char *env = std::getenv(name);
    if (!env) return dflt;
    const int v = std::atoi(env);
    return v >= 1 && v <= (int)kStreamMax ? (uint32_t)v : dflt;
}


hpss_status stream_line_and_search(hpss_handle h, const float *samples, const float *m0s,
                                   uint32_t nM0, const uint32_t *granularity, int kernel,
                                   float *out, hpss_stats *stats) {
    if (!h->copyStream)
        HPSS_CUDA_TRY(h, cudaStreamCreateWithFlags(&h->copyStream, cudaStreamNonBlocking));
    const uint32_t nChunks = stream_count("HPSS_STREAM_CHUNKS", kStreamChunks);
    const uint32_t nGroups = stream_count("HPSS_STREAM_GROUPS", kStreamGroups);
    while (h->streamEvents.size() < nChunks + nGroups) {
        cudaEvent_t e;
        HPSS_CUDA_TRY(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        h->streamEvents.push_back(e);
    }
    if (!h->streamT0) HPSS_CUDA_TRY(h, cudaEventCreate(&h->streamT0));
    if (!h->streamT1) HPSS_CUDA_TRY(h, cudaEventCreate(&h->streamT1));
    cudaEvent_t *chunkDone = h->streamEvents.data();
    cudaEvent_t *groupDone = chunkDone + nChunks;
    const uint32_t n = h->nTraces;
    uint32_t bound[kStreamMax + 1];
    for (uint32_t k = 0; k <= nChunks; k++)
        bound[k] = (uint32_t)((uint64_t)n * k / nChunks);
    if (n && h->stride != h->S && h->storage == HPSS_STORAGE_FP32)
        HPSS_CUDA_TRY(h, cudaMemsetAsync(h->dSamples, 0, (size_t)n * h->stride * sizeof(float),
                                         h->copyStream));
    for (uint32_t k = 0; k < nChunks; k++) {
        HPSS_CUDA_TRY(h, copy_line_rows(h, samples, bound[k], bound[k + 1], h->copyStream));
        HPSS_CUDA_TRY(h, cudaEventRecord(chunkDone[k], h->copyStream));
    }
    // every search below waits for the chunks it reads
    h->gatherReady = true;
    if (nM0 == 0) {
        HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->copyStream));
        HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        release_upload_staging(h);
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return HPSS_OK;
    }
    const size_t block = (size_t)(2 + h->np) * h->S;
    HPSS_CUDA_TRY(h, ensure(h, h->m0s, nM0 * sizeof(float)));
    HPSS_CUDA_TRY(h, ensure(h, h->out, nM0 * block * sizeof(float)));
    HPSS_CUDA_TRY(h, ensure(h, h->notUsed, 16 + nM0 * sizeof(unsigned long long)));
    HPSS_CUDA_TRY(h, cudaMemcpyAsync(h->m0s.p, m0s, nM0 * sizeof(float),
                                     cudaMemcpyHostToDevice, h->stream));
    HPSS_CUDA_TRY(h, cudaMemsetAsync(h->notUsed.p, 0, 16 + nM0 * sizeof(unsigned long long),
                                     h->stream));
    HPSS_CUDA_TRY(h, cudaEventRecord(h->streamT0, h->stream));
    // midpoint distance within which a trace can be selected, widened so that
    // a group never starts before its traces have arrived
    float hmax = 0.f;
    for (float v : h->hHoff) hmax = std::max(hmax, std::fabs(v));
    const float radius = h->model == HPSS_MODEL_CMP ? 0.f
                         : h->model == HPSS_MODEL_ZOCRS
                             ? h->apm
                             : h->apm + std::sqrt(hmax * hmax + h->h0 * h->h0);
    // groups of ceil(nM0 / nGroups) midpoints, the last one smaller: the
    // first group is the largest, so the per-call buffers the search grows
    // (selection, candidate parts) are sized by it and never reallocated
    // under a later group's launches
    const uint32_t per = (nM0 + nGroups - 1) / nGroups;
    const uint32_t G = (nM0 + per - 1) / per;
    auto first = [&](uint32_t g) { return std::min(g * per, nM0); };
    auto back = [&](uint32_t g) -> cudaError_t {
        cudaError_t e = cudaStreamWaitEvent(h->copyStream, groupDone[g], 0);
        if (e != cudaSuccess) return e;
        const size_t i0 = first(g), cnt = first(g + 1) - i0;
        return cudaMemcpyAsync(out + i0 * block, static_cast<float *>(h->out.p) + i0 * block,
                               cnt * block * sizeof(float), cudaMemcpyDeviceToHost,
                               h->copyStream);
    };
    for (uint32_t g = 0; g < G; g++) {
        const uint32_t i0 = first(g), i1 = first(g + 1);
        size_t need = 0;
        for (uint32_t i = i0; i < i1 && need < n; i++) {
            const float m0 = m0s[i];
            if (!std::isfinite(m0)) {
                need = n;
                break;
            }
            const float reach = m0 + radius + 1e-3f * (std::fabs(m0) + radius) + 1.f;
            need = std::max<size_t>(
                need, std::upper_bound(h->hMid.begin(), h->hMid.end(), reach) - h->hMid.begin());
        }
        if (need > 0) {
            uint32_t k = 0;
            while (bound[k + 1] < need) k++;
            HPSS_CUDA_TRY(h, cudaStreamWaitEvent(h->stream, chunkDone[k], 0));
        }
        const GroupOfCall grp{i0};
        hpss_status rc = linear_search_impl(h, static_cast<float *>(h->m0s.p) + i0, i1 - i0,
                                            granularity, kernel,
                                            static_cast<float *>(h->out.p) + i0 * block, nullptr,
                                            false, &grp);
        if (rc != HPSS_OK) return rc;
        HPSS_CUDA_TRY(h, cudaEventRecord(groupDone[g], h->stream));
        // the previous group's results return while this group runs
        if (g > 0) HPSS_CUDA_TRY(h, back(g - 1));
    }
    HPSS_CUDA_TRY(h, cudaEventRecord(h->streamT1, h->stream));
    HPSS_CUDA_TRY(h, back(G - 1));
    HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->copyStream));
    HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    release_upload_staging(h);
    const char *counters = static_cast<const char *>(h->notUsed.p);
    uint32_t err = 0;
    unsigned long long ties = 0;
    HPSS_CUDA_TRY(h, cudaMemcpy(&err, counters, sizeof(err), cudaMemcpyDeviceToHost));
    HPSS_CUDA_TRY(h, cudaMemcpy(&ties, counters + 8, sizeof(ties), cudaMemcpyDeviceToHost));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        // selected traces of every midpoint, for the evaluation count
        LsParams lp;
        fill_line_params(h, lp);
        lp.m0s = static_cast<float *>(h->m0s.p);
        lp.nM0 = nM0;
        hpss_status rc = run_selection(h, lp.m0s, nM0, lp);
        if (rc != HPSS_OK) return rc;
        std::vector<uint32_t> cnt(nM0);
        std::vector<unsigned long long> nu(nM0);
        HPSS_CUDA_TRY(h, cudaMemcpyAsync(cnt.data(), lp.selCount, nM0 * sizeof(uint32_t),
                                         cudaMemcpyDeviceToHost, h->stream));
        HPSS_CUDA_TRY(h, cudaMemcpyAsync(nu.data(), counters + 16,
                                         nM0 * sizeof(unsigned long long),
                                         cudaMemcpyDeviceToHost, h->stream));
        HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        double P = 1, sel = 0, nus = 0;
        for (uint32_t j = 0; j < h->np; j++) P *= granularity[j];
        for (uint32_t i = 0; i < nM0; i++) {
            sel += cnt[i];
            nus += (double)nu[i];
        }
        stats->selected_traces = sel;
        stats->evals = sel * (double)h->S * P;
        stats->not_used = nus;
        float ms = 0;
        cudaEventElapsedTime(&ms, h->streamT0, h->streamT1);
        stats->kernel_ms = ms;
        stats->device_error = err;
        stats->kernel_variant = h->lastVariant;
        stats->near_ties = (double)ties;
        stats->candidate_parts = h->lastParts;
    }
    if (err)
        return set_error(h, HPSS_ERR_DEVICE_CHECK,
                         "device check failed, error word " + std::to_string(err));
    return HPSS_OK;
}

}  // namespace hpss
