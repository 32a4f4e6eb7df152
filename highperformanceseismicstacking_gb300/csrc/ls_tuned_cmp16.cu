// ls_tuned_cmp16.cu -- tuned linear-search kernel instantiations for the
// CMP traveltime model over 16-bit rows staged by bulk copies and widened
// in shared memory (S16; kernel body in ls_tuned.cuh), stack from the
// per-tap sums.
#include "ls_tuned.cuh"

namespace hpss {

cudaError_t launch_ls_tuned_cmp16(const LsParams &p, uint32_t grid, uint32_t tiles,
                                 uint32_t nUnits, cudaStream_t st, int variant) {
    if (variant == 1)
        return launch_ls_tuned2_model<kModelCmp, 1, 3, false, 0, true>(p, grid, tiles, nUnits, st);
    if (variant == 2)
        return launch_ls_tuned2_model<kModelCmp, 2, 3, false, 0, true>(p, grid, tiles, nUnits, st);
    return launch_ls_tuned2_model<kModelCmp, 2, 2, false, 0, true>(p, grid, tiles, nUnits, st);
}

}  // namespace hpss
