// Fused Heun step kernels (llg_fused.cuh) of the simple-cubic and bcc
// nearest-neighbour families, the fused tile rows of every family, and the
// launcher; llg_fused_b.cu compiles the other families in parallel.
#include "llg_fused.cuh"

namespace jams_llg {

cudaError_t launch_fused_b(int family, bool wide, int occupancy, unsigned grid, cudaStream_t st, const Params& P,
                           const TiledParams& TP, const float* s0, float* s1, uint32_t k, uint32_t adv);

bool fused_supported(int family) {
  return family == kFamSC || family == kFamBCC || family == kFamBCC3 || family == kFamFCC || family == kFamFCC2;
}

// tile rows of the fused kernel: a wide and a narrow variant per family (the
// halo cells a tile recomputes cost less on a wide tile; a narrow one gives
// more CTAs and more resident CTAs per SM)
int fused_rows(int family, bool wide) {
  switch (family) {
    case kFamSC: return wide ? 16 : 8;
    case kFamBCC:
    case kFamBCC3: return wide ? 8 : 4;
    case kFamFCC:
    case kFamFCC2: return 4;
    default: return 0;
  }
}

cudaError_t launch_fused(int family, bool wide, int occupancy, unsigned grid, cudaStream_t st, const Params& P,
                         const TiledParams& TP, const float* s0, float* s1, uint32_t k, uint32_t adv) {
  switch (family) {
    case kFamSC:
      return wide ? launch_fused_occ<FamSC, 16>(occupancy, grid, st, P, TP, s0, s1, k, adv)
                  : launch_fused_occ<FamSC, 8>(occupancy, grid, st, P, TP, s0, s1, k, adv);
    case kFamBCC:
      return wide ? launch_fused_occ<FamBCC, 8>(occupancy, grid, st, P, TP, s0, s1, k, adv)
                  : launch_fused_occ<FamBCC, 4>(occupancy, grid, st, P, TP, s0, s1, k, adv);
    default:
      return launch_fused_b(family, wide, occupancy, grid, st, P, TP, s0, s1, k, adv);
  }
}

}  // namespace jams_llg
