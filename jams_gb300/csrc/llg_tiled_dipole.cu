// Tiled FP32 stage kernels (llg_tiled.cuh) of models with a dipole term: the
// same kernels reading the precomputed dipole field planes.
#include "llg_tiled.cuh"

namespace jams_llg {

template cudaError_t launch_tiled_t<true, 1, false>(int, int, int, int, unsigned, cudaStream_t, const Params&,
                                                    const TiledParams&, const float*, const float*, float*, float*,
                                                    uint32_t, uint32_t, const CUtensorMap*);

}  // namespace jams_llg
