// Tiled FP32 stage kernels (llg_tiled.cuh) of simple-cubic models on the
// half-width tile: 16 cells along z by 8 rows, one or two rows per thread.
// A lattice whose z extent is not a multiple of 32 leaves fewer lanes idle
// on it (replica sweeps of edges 16..64: 82 % of the lanes busy against
// 76 % on the 32-cell tile).  Compiled in parallel with the other tiles.
#include "llg_tiled.cuh"

namespace jams_llg {

cudaError_t launch_tiled_sc16(int rpt, int occupancy, int stage, unsigned grid, cudaStream_t st, const Params& P,
                              const TiledParams& TP, const float* s0, const float* sin, float* out, float* aux,
                              uint32_t k, uint32_t adv) {
  if (rpt == 2)
    return launch_occ<FamSC, 16, 8, 2, false, false>(occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv,
                                                     nullptr);
  return launch_occ<FamSC, 16, 8, 1, false, false>(occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv,
                                                   nullptr);
}

}  // namespace jams_llg
