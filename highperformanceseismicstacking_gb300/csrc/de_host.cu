// de_host.cu -- host side of the differential evolution behind the C ABI:
// selection (CMP / ZO-CRS as the linear search, OCT from the initial
// population), the work-queue order and the fused DE launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "hpss_handle.h"

namespace hpss {

hpss_status de_impl(hpss_handle h, const float *d_m0s, uint32_t nM0, uint32_t pop,
                    uint32_t gens, float F, float CR, uint64_t seed, float *d_out,
                    hpss_stats *stats, bool sync) {
    hpss_status rc = check_ready(h);
    if (rc != HPSS_OK) return rc;
    if (pop < 1 || pop > kDeMaxPopulation)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "population must be in [1, 128]");
    if (gens < 1) return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "generations must be >= 1");
    if (nM0 == 0) return HPSS_OK;
    if (!d_m0s || !d_out) return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "null device pointer");
    cudaSetDevice(h->device);

    DeParams d{};
    fill_line_params(h, d.ls);
    d.ls.m0s = d_m0s;
    d.ls.nM0 = nM0;
    d.ls.out = d_out;
    HPSS_CUDA_TRY(h, use_oct_table(h, d.ls));
    // OCT over several half-offsets: the midpoints in h0 blocks, one launch
    // over all of them (the random stream is keyed by the midpoint's value,
    // so block b equals a one-h0 call at h0s[b])
    HPSS_CUDA_TRY(h, expand_h0_blocks(h, d.ls));
    d_m0s = d.ls.m0s;
    nM0 = d.ls.nM0;
    d.pop = pop;
    d.gens = gens;
    d.F = F;
    d.CR = CR;
    d.seedLo = (uint32_t)seed;
    d.seedHi = (uint32_t)(seed >> 32);
    for (int j = 0; j < 3; j++) {
        d.lo[j] = h->lower[j];
        d.hi[j] = h->upper[j];
    }
    HPSS_CUDA_TRY(h, ensure(h, h->notUsed, nM0 * sizeof(unsigned long long)));
    // error word at byte 0, the DE kernel's work-queue counter at byte 8
    HPSS_CUDA_TRY(h, ensure(h, h->errWord, 16));
    d.ls.notUsed = static_cast<unsigned long long *>(h->notUsed.p);
    d.ls.errorWord = static_cast<uint32_t *>(h->errWord.p);
    d.ls.unitCounter = reinterpret_cast<uint32_t *>(static_cast<char *>(h->errWord.p) + 8);
    HPSS_CUDA_TRY(h, cudaMemsetAsync(d.ls.notUsed, 0, nM0 * sizeof(unsigned long long), h->stream));
    HPSS_CUDA_TRY(h, cudaMemsetAsync(h->errWord.p, 0, 16, h->stream));
    const bool ordered = nM0 > 1 && nM0 <= kMaxOrderedMidpoints;
    if (ordered) HPSS_CUDA_TRY(h, ensure(h, h->order, nM0 * sizeof(uint32_t)));

    HPSS_CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream));
    // selection: CMP / ZO-CRS as linear search; OCT with the initial population
    HPSS_CUDA_TRY(h, ensure(h, h->selFirst, nM0 * sizeof(uint32_t)));
    HPSS_CUDA_TRY(h, ensure(h, h->selCount, nM0 * sizeof(uint32_t)));
    d.ls.selFirst = static_cast<uint32_t *>(h->selFirst.p);
    d.ls.selCount = static_cast<uint32_t *>(h->selCount.p);
    d.ls.selIdx = nullptr;
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
        d.ls.selIdx = static_cast<uint32_t *>(h->selIdx.p);
        HPSS_CUDA_TRY(h, ensure(h, h->deBoxes, (size_t)nM0 * h->S * sizeof(float4)));
        HPSS_CUDA_TRY(h, launch_de_select_oct(d, cf, cc, static_cast<uint32_t *>(h->selIdx.p),
                                              static_cast<uint32_t *>(h->selCount.p),
                                              (uint64_t)total,
                                              static_cast<float4 *>(h->deBoxes.p), h->stream));
    }
    // work queue order: midpoints by descending selected traces
    if (ordered) {
        HPSS_CUDA_TRY(h, launch_order_by_count(d.ls.selCount, nM0,
                                               static_cast<uint32_t *>(h->order.p), h->stream));
        d.ls.order = static_cast<const uint32_t *>(h->order.p);
    }
    HPSS_CUDA_TRY(h, cudaEventRecord(h->ev1, h->stream));
    const uint64_t units = (uint64_t)nM0 * h->S;
    // unit indices (and a work-queue counter past the last unit) stay below 2^31
    if (units > 0x7fffffffull)
        return set_error(h, HPSS_ERR_INVALID_ARGUMENT, "too many (midpoint, sample) units");
    HPSS_CUDA_TRY(h, launch_de(d, h->model, (uint32_t)num_sms(h), h->stream));
    HPSS_CUDA_TRY(h, cudaEventRecord(h->ev2, h->stream));
    if (stats || sync) {
        HPSS_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        uint32_t err = 0;
        HPSS_CUDA_TRY(h, cudaMemcpy(&err, d.ls.errorWord, sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost));
        if (stats) {
            std::memset(stats, 0, sizeof(*stats));
            std::vector<uint32_t> cnt(nM0);
            std::vector<unsigned long long> nu(nM0);
            HPSS_CUDA_TRY(h, cudaMemcpy(cnt.data(), d.ls.selCount, nM0 * sizeof(uint32_t),
                                        cudaMemcpyDeviceToHost));
            HPSS_CUDA_TRY(h, cudaMemcpy(nu.data(), d.ls.notUsed,
                                        nM0 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
            double sel = 0, nus = 0;
            for (uint32_t i = 0; i < nM0; i++) {
                sel += cnt[i];
                nus += (double)nu[i];
            }
            stats->selected_traces = sel;
            stats->evals = sel * (double)h->S * (double)pop * (double)gens;
            stats->not_used = nus;
            float ms = 0;
            cudaEventElapsedTime(&ms, h->ev1, h->ev2);
            stats->kernel_ms = ms;
            cudaEventElapsedTime(&ms, h->ev0, h->ev1);
            stats->selection_ms = ms;
            stats->kernel_variant = -1;
            stats->device_error = err;
        }
        if (err & kErrTimeout)
            return set_error(h, HPSS_ERR_TIMEOUT,
                             "staging copies did not complete in time, error word " +
                                 std::to_string(err));
    }
    return HPSS_OK;
}

}  // namespace hpss
