// Tiled FP32 stage kernels (llg_tiled.cuh) with TMA plane loads and two rows
// per thread: compiled in parallel with the others.
#include "llg_tiled.cuh"

namespace jams_llg {

template cudaError_t launch_tiled_t<false, 2, true>(int, int, int, int, unsigned, cudaStream_t, const Params&,
                                                    const TiledParams&, const float*, const float*, float*, float*,
                                                    uint32_t, uint32_t, const CUtensorMap*);

}  // namespace jams_llg
