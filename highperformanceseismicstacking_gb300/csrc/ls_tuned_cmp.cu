// ls_tuned_cmp.cu -- tuned linear-search kernel instantiations for the
// CMP traveltime model, stack from the per-tap sums (kernel body in
// ls_tuned.cuh; the EXACT_STACK instantiations are in ls_tuned_cmp_exact.cu).
#include "ls_tuned.cuh"

namespace hpss {

cudaError_t launch_ls_tuned_cmp(const LsParams &p, uint32_t grid, uint32_t tiles,
                                uint32_t nUnits, cudaStream_t st, int variant,
                                bool exactStack) {
    if (exactStack) return launch_ls_tuned_cmp_exact(p, grid, tiles, nUnits, st, variant);
    if (p.samples16) return launch_ls_tuned_cmp16(p, grid, tiles, nUnits, st, variant);
    if (variant == 1) return launch_ls_tuned2_model<kModelCmp, 1, 3, false>(p, grid, tiles, nUnits, st);
    if (variant == 2) return launch_ls_tuned2_model<kModelCmp, 2, 3, false>(p, grid, tiles, nUnits, st);
    return launch_ls_tuned2_model<kModelCmp, 2, 2, false>(p, grid, tiles, nUnits, st);
}

// staged floats per CTA of the largest (2 CTAs/SM) and smallest (3 CTAs/SM)
// shapes: a trace row must fit the stage
size_t tuned_stage_floats() { return Stage2<2>::kFloats; }
size_t tuned_stage_floats_min() { return Stage2<3>::kFloats; }

}  // namespace hpss
