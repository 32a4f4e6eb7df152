// ls_tuned_prec.cu -- tuned linear-search kernel instantiations with the
// precision modes (kernel body in ls_tuned.cuh): CMP with compensated window
// sums; ZO-CRS with the FP64 traveltime, compensated sums or both.  One
// shape (one candidate pair per thread, 3 CTAs per SM): the compensated
// totals take registers the two-pair shapes do not have.
#include "ls_tuned.cuh"

namespace hpss {

cudaError_t launch_ls_tuned_prec(const LsParams &p, int model, int prec, uint32_t grid,
                                 uint32_t tiles, uint32_t nUnits, cudaStream_t st) {
    constexpr int C = kPrecCompensated, T = kPrecTt64;
    if (model == kModelCmp) {
        // the CMP time has no FP64 form: only the compensated sums apply
        if (prec & C) return launch_ls_tuned2_model<kModelCmp, 1, 3, false, C>(p, grid, tiles, nUnits, st);
        return launch_ls_tuned2_model<kModelCmp, 1, 3, false, 0>(p, grid, tiles, nUnits, st);
    }
    if (model != kModelZocrs) return cudaErrorNotSupported;
    switch (prec & (C | T)) {
        case T: return launch_ls_tuned2_model<kModelZocrs, 1, 3, false, T>(p, grid, tiles, nUnits, st);
        case C: return launch_ls_tuned2_model<kModelZocrs, 1, 3, false, C>(p, grid, tiles, nUnits, st);
        case C | T:
            return launch_ls_tuned2_model<kModelZocrs, 1, 3, false, C | T>(p, grid, tiles, nUnits, st);
        default: return launch_ls_tuned2_model<kModelZocrs, 1, 3, false, 0>(p, grid, tiles, nUnits, st);
    }
}

}  // namespace hpss
