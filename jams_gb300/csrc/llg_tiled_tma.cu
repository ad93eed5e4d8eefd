// Tiled FP32 stage kernels (llg_tiled.cuh) whose planes arrive by TMA box
// loads, one row per thread (models without a dipole term, one replica):
// compiled in parallel with the register-staged kernels.
#include "llg_tiled.cuh"

namespace jams_llg {

template cudaError_t launch_tiled_t<false, 1, true>(int, int, int, int, unsigned, cudaStream_t, const Params&,
                                                    const TiledParams&, const float*, const float*, float*, float*,
                                                    uint32_t, uint32_t, const CUtensorMap*);

}  // namespace jams_llg
