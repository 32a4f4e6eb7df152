// ls_tuned_zocrs.cu -- tuned linear-search kernel instantiations for the
// ZOCRS traveltime model (kernel body in ls_tuned.cuh).
#include "ls_tuned.cuh"

namespace hpss {

cudaError_t launch_ls_tuned_zocrs(const LsParams &p, uint32_t grid, uint32_t tiles,
                                uint32_t nUnits, cudaStream_t st) {
    return launch_ls_tuned_model<kModelZocrs, 4>(p, grid, tiles, nUnits, st);
}

}  // namespace hpss
