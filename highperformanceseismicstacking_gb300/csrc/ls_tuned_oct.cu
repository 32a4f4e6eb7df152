// ls_tuned_oct.cu -- tuned linear-search kernel instantiations for the
// OCT traveltime model (kernel body in ls_tuned.cuh).
#include "ls_tuned.cuh"

namespace hpss {

cudaError_t launch_ls_tuned_oct(const LsParams &p, uint32_t grid, uint32_t tiles,
                                uint32_t nUnits, cudaStream_t st, int) {
    return launch_ls_tuned_model<kModelOct, 4>(p, grid, tiles, nUnits, st);
}

}  // namespace hpss
