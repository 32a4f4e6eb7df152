// ls_tuned_cmp.cu -- tuned linear-search kernel instantiations for the
// CMP traveltime model (kernel body in ls_tuned.cuh).
#include "ls_tuned.cuh"

namespace hpss {

// pairs: candidate pairs per thread (chunk = 8 warps x 2*pairs candidates)
cudaError_t launch_ls_tuned_cmp(const LsParams &p, uint32_t grid, uint32_t tiles,
                                uint32_t nUnits, cudaStream_t st, int pairs) {
    if (pairs == 1) return launch_ls_tuned2_model<kModelCmp, 1>(p, grid, tiles, nUnits, st);
    if (pairs == 4) return launch_ls_tuned2_model<kModelCmp, 4>(p, grid, tiles, nUnits, st);
    return launch_ls_tuned2_model<kModelCmp, 2>(p, grid, tiles, nUnits, st);
}

size_t tuned_smem_bytes() { return sizeof(TunedSmem); }
size_t tuned_stage_floats() { return kStageFloats; }

}  // namespace hpss
