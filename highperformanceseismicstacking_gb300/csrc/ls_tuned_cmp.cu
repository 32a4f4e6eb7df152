// ls_tuned_cmp.cu -- tuned linear-search kernel instantiations for the
// CMP traveltime model (kernel body in ls_tuned.cuh).
#include "ls_tuned.cuh"

namespace hpss {

// variant: 0 = 2 candidate pairs per thread, 2 CTAs/SM; 1 = 1 pair, 3 CTAs/SM;
// 2 = 2 pairs, 3 CTAs/SM (chunk = 8 warps x 2*pairs candidates)
cudaError_t launch_ls_tuned_cmp(const LsParams &p, uint32_t grid, uint32_t tiles,
                                uint32_t nUnits, cudaStream_t st, int variant) {
    if (variant == 1) return launch_ls_tuned2_model<kModelCmp, 1, 3>(p, grid, tiles, nUnits, st);
    if (variant == 2) return launch_ls_tuned2_model<kModelCmp, 2, 3>(p, grid, tiles, nUnits, st);
    return launch_ls_tuned2_model<kModelCmp, 2, 2>(p, grid, tiles, nUnits, st);
}

size_t tuned_smem_bytes() { return sizeof(TunedSmem); }
size_t tuned_stage_floats() { return kStageFloats; }
size_t tuned_stage_floats_min() { return Stage2<3>::kFloats; }

}  // namespace hpss
