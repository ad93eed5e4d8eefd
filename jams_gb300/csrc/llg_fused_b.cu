// Fused Heun step kernels (llg_fused.cuh) of the bcc three-shell and fcc
// families (compiled apart from llg_fused_a.cu, in parallel).
#include "llg_fused.cuh"

namespace jams_llg {

cudaError_t launch_fused_b(int family, bool wide, int occupancy, unsigned grid, cudaStream_t st, const Params& P,
                           const TiledParams& TP, const float* s0, float* s1, uint32_t k, uint32_t adv) {
  switch (family) {
    case kFamBCC3:
      return wide ? launch_fused_occ<FamBCC3, 8>(occupancy, grid, st, P, TP, s0, s1, k, adv)
                  : launch_fused_occ<FamBCC3, 4>(occupancy, grid, st, P, TP, s0, s1, k, adv);
    case kFamFCC: return launch_fused_occ<FamFCC, 4>(occupancy, grid, st, P, TP, s0, s1, k, adv);
    case kFamFCC2: return launch_fused_occ<FamFCC2, 4>(occupancy, grid, st, P, TP, s0, s1, k, adv);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace jams_llg
