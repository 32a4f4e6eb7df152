// ls_tuned_zocrs.cu -- tuned linear-search kernel instantiations for the
// ZO-CRS traveltime model, stack from the per-tap sums (kernel body in
// ls_tuned.cuh; the EXACT_STACK instantiations are in ls_tuned_zocrs_exact.cu).
#include "ls_tuned.cuh"

namespace hpss {

cudaError_t launch_ls_tuned_zocrs(const LsParams &p, uint32_t grid, uint32_t tiles,
                                uint32_t nUnits, cudaStream_t st, int variant,
                                bool exactStack) {
    if (exactStack) return launch_ls_tuned_zocrs_exact(p, grid, tiles, nUnits, st, variant);
    if (p.samples16) return launch_ls_tuned_zocrs16(p, grid, tiles, nUnits, st, variant);
    if (variant == 1) return launch_ls_tuned2_model<kModelZocrs, 1, 3, false>(p, grid, tiles, nUnits, st);
    if (variant == 2) return launch_ls_tuned2_model<kModelZocrs, 2, 3, false>(p, grid, tiles, nUnits, st);
    return launch_ls_tuned2_model<kModelZocrs, 2, 2, false>(p, grid, tiles, nUnits, st);
}

}  // namespace hpss
