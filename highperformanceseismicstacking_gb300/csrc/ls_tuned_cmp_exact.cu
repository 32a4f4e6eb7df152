// ls_tuned_cmp_exact.cu -- tuned linear-search kernel instantiations for
// the CMP traveltime model with the linear sum accumulated in the
// reference's order (EXACT_STACK; kernel body in ls_tuned.cuh).
#include "ls_tuned.cuh"

namespace hpss {

cudaError_t launch_ls_tuned_cmp_exact(const LsParams &p, uint32_t grid, uint32_t tiles,
                                      uint32_t nUnits, cudaStream_t st, int variant) {
    if (variant == 1) return launch_ls_tuned2_model<kModelCmp, 1, 3, true>(p, grid, tiles, nUnits, st);
    if (variant == 2) return launch_ls_tuned2_model<kModelCmp, 2, 3, true>(p, grid, tiles, nUnits, st);
    return launch_ls_tuned2_model<kModelCmp, 2, 2, true>(p, grid, tiles, nUnits, st);
}

}  // namespace hpss
