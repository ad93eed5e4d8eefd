// Tiled FP32 stage kernels (llg_tiled.cuh) of models without a dipole term,
// the tile geometry of each family, and the launcher for both variants.
#include "llg_tiled.cuh"

namespace jams_llg {

template cudaError_t launch_tiled_t<false, 1, false>(int, int, int, int, unsigned, cudaStream_t, const Params&,
                                                     const TiledParams&, const float*, const float*, float*, float*,
                                                     uint32_t, uint32_t, const CUtensorMap*);
extern template cudaError_t launch_tiled_t<true, 1, false>(int, int, int, int, unsigned, cudaStream_t, const Params&,
                                                           const TiledParams&, const float*, const float*, float*,
                                                           float*, uint32_t, uint32_t, const CUtensorMap*);
extern template cudaError_t launch_tiled_t<false, 2, false>(int, int, int, int, unsigned, cudaStream_t, const Params&,
                                                            const TiledParams&, const float*, const float*, float*,
                                                            float*, uint32_t, uint32_t, const CUtensorMap*);
extern template cudaError_t launch_tiled_t<false, 1, true>(int, int, int, int, unsigned, cudaStream_t, const Params&,
                                                           const TiledParams&, const float*, const float*, float*,
                                                           float*, uint32_t, uint32_t, const CUtensorMap*);
extern template cudaError_t launch_tiled_t<false, 2, true>(int, int, int, int, unsigned, cudaStream_t, const Params&,
                                                           const TiledParams&, const float*, const float*, float*,
                                                           float*, uint32_t, uint32_t, const CUtensorMap*);

void tiled_geometry(int family, int* tz, int* ty) {
  switch (family) {
    case kFamSC: *tz = 32; *ty = 8; break;
    case kFamBCC:
    case kFamBCC3: *tz = 32; *ty = 4; break;
    case kFamTRI: *tz = 256; *ty = 1; break;
    case kFamFCC:
    case kFamFCC2: *tz = 32; *ty = 2; break;
    default: *tz = 0; *ty = 0; break;
  }
}

// rows of the narrow tile variant of a family (the wide one when it has none)
int narrow_tile_rows(int family) {
  if (family == kFamSC) return 4;
  int tz, ty;
  tiled_geometry(family, &tz, &ty);
  return ty;
}

bool pair_rows_supported(int family) {
  return family == kFamSC || family == kFamBCC || family == kFamBCC3 || family == kFamFCC || family == kFamFCC2;
}

cudaError_t launch_tiled_sc16(int rpt, int occupancy, int stage, unsigned grid, cudaStream_t st, const Params& P,
                              const TiledParams& TP, const float* s0, const float* sin, float* out, float* aux,
                              uint32_t k, uint32_t adv);

cudaError_t launch_tiled(int family, int tz, int ty, int rpt, int occupancy, int stage, unsigned grid,
                         cudaStream_t st, const Params& P, const TiledParams& TP, const float* s0, const float* sin,
                         float* out, float* aux, uint32_t k, uint32_t advance, bool dipole, const CUtensorMap* map) {
  if (tz == 16) {   // the half-width simple-cubic tile (llg_tiled_z16.cu)
    if (family != kFamSC || ty != 8 || dipole || map) return cudaErrorInvalidValue;
    return launch_tiled_sc16(rpt, occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, advance);
  }
  if (dipole) {
    if (rpt != 1 || map) return cudaErrorInvalidValue;
    return launch_tiled_t<true, 1, false>(family, ty, occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, advance,
                                          nullptr);
  }
  if (map) {
    if (rpt == 2)
      return launch_tiled_t<false, 2, true>(family, ty, occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k,
                                            advance, map);
    return launch_tiled_t<false, 1, true>(family, ty, occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, advance,
                                          map);
  }
  if (rpt == 2)
    return launch_tiled_t<false, 2, false>(family, ty, occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k,
                                           advance, nullptr);
  return launch_tiled_t<false, 1, false>(family, ty, occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, advance,
                                         nullptr);
}

// box geometry of the TMA plane loads of a family's tile (TmaGeo): element
// offset before z0 - RZ, box width in elements, rows; false where the
// tiles are not 32 cells wide
bool tma_box(int family, int ty, int* lo, int* width, int* rows) {
  switch (family) {
    case kFamSC:
      if (ty == 4) return *lo = TmaGeo<FamSC, 32, 4>::LO, *width = TmaGeo<FamSC, 32, 4>::BW,
                          *rows = TmaGeo<FamSC, 32, 4>::ROWS, true;
      return *lo = TmaGeo<FamSC, 32, 8>::LO, *width = TmaGeo<FamSC, 32, 8>::BW, *rows = TmaGeo<FamSC, 32, 8>::ROWS,
             true;
    case kFamBCC:
    case kFamBCC3:
      return *lo = TmaGeo<FamBCC, 32, 4>::LO, *width = TmaGeo<FamBCC, 32, 4>::BW, *rows = TmaGeo<FamBCC, 32, 4>::ROWS,
             true;
    case kFamFCC:
    case kFamFCC2:
      return *lo = TmaGeo<FamFCC, 32, 2>::LO, *width = TmaGeo<FamFCC, 32, 2>::BW, *rows = TmaGeo<FamFCC, 32, 2>::ROWS,
             true;
    default: return false;
  }
}

}  // namespace jams_llg
