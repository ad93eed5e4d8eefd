// Tiled FP32 stage kernels (llg_tiled.cuh) with two rows per thread, for
// models without a dipole term: compiled in parallel with the one-row
// kernels.
#include "llg_tiled.cuh"

namespace jams_llg {

template cudaError_t launch_tiled_t<false, 2, false>(int, int, int, int, unsigned, cudaStream_t, const Params&,
                                                     const TiledParams&, const float*, const float*, float*, float*,
                                                     uint32_t, uint32_t, const CUtensorMap*);

}  // namespace jams_llg
