// ls_tuned_zocrs.cu -- tuned linear-search kernel instantiations for the
// ZOCRS traveltime model (kernel body in ls_tuned.cuh).
#include "ls_tuned.cuh"

namespace hpss {

// variant: 0 = 2 candidate pairs per thread, 2 CTAs/SM; 1 = 1 pair, 3 CTAs/SM;
// 2 = 2 pairs, 3 CTAs/SM (chunk = 8 warps x 2*pairs candidates)
cudaError_t launch_ls_tuned_zocrs(const LsParams &p, uint32_t grid, uint32_t tiles,
                                uint32_t nUnits, cudaStream_t st, int variant) {
    if (variant == 1) return launch_ls_tuned2_model<kModelZocrs, 1, 3>(p, grid, tiles, nUnits, st);
    if (variant == 2) return launch_ls_tuned2_model<kModelZocrs, 2, 3>(p, grid, tiles, nUnits, st);
    return launch_ls_tuned2_model<kModelZocrs, 2, 2>(p, grid, tiles, nUnits, st);
}

}  // namespace hpss
