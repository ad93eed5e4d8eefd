// Declarations of the kernels in llg_kernels.cu, launched by llg_host.cu.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "llg_internal.h"

namespace jams_llg {

__global__ void heun_predict_f32(const __grid_constant__ Params P, const float* __restrict__ s0,
                                 float* __restrict__ sp, float* __restrict__ rhs0, uint32_t kstep);
__global__ void heun_correct_f32(const __grid_constant__ Params P, const float* __restrict__ s0,
                                 const float* __restrict__ sp, float* __restrict__ s1,
                                 const float* __restrict__ rhs0, uint32_t kstep);
__global__ void heun_predict_f64(const __grid_constant__ Params P, const double* __restrict__ s0,
                                 double* __restrict__ sp, double* __restrict__ ds, uint32_t kstep);
__global__ void heun_correct_f64(const __grid_constant__ Params P, const double* s0, const double* sp,
                                 const double* ds, double* s1, uint32_t kstep);
template <int STAGE>
__global__ void rk4_stage_f32(const __grid_constant__ Params P, const float* s0, const float* sin, float* acc,
                              float* sout, uint32_t kstep);
template <int STAGE>
__global__ void rk4_stage_f64(const __grid_constant__ Params P, const double* s0, const double* sin,
                              double* acc, double* sout, uint32_t kstep);
__global__ void advance_step_base(uint64_t* base, uint32_t nsteps);
template <typename Real>
__global__ void unpack_state(const double* __restrict__ aos, Real* __restrict__ soa, int64_t offset, int64_t n,
                             int64_t npad);
template <typename Real>
__global__ void pack_state(const Real* __restrict__ soa, double* __restrict__ aos, int64_t offset, int64_t n,
                           int64_t npad);
__global__ void fields_f32(const __grid_constant__ Params P, const float* __restrict__ s0,
                           double* __restrict__ out, int replica);
__global__ void fields_f64(const __grid_constant__ Params P, const double* __restrict__ s0,
                           double* __restrict__ out, int replica);
__global__ void term_fields_f32(const __grid_constant__ Params P, const float* __restrict__ s0,
                                double* __restrict__ out, int replica, int term);
__global__ void term_fields_f64(const __grid_constant__ Params P, const double* __restrict__ s0,
                                double* __restrict__ out, int replica, int term);

void launch_rk4_f32(int stage, unsigned grid, cudaStream_t st, const Params& P, const float* s0, const float* sin,
                    float* acc, float* sout, uint32_t k);
void launch_rk4_f64(int stage, unsigned grid, cudaStream_t st, const Params& P, const double* s0,
                    const double* sin, double* acc, double* sout, uint32_t k);
void launch_unpack(bool fp64, cudaStream_t st, const double* aos, void* soa, int64_t offset, int64_t n,
                   int64_t npad);
void launch_pack(bool fp64, cudaStream_t st, const void* soa, double* aos, int64_t offset, int64_t n,
                 int64_t npad);

// tiled FP32 kernels (llg_tiled.cuh, instantiated by llg_tiled*.cu); family ids in llg_families.h
void tiled_geometry(int family, int* tz, int* ty);
// ty: tile rows (the family's wide tile from tiled_geometry or the narrow
// one from narrow_tile_rows); rpt: rows per thread, 1 or 2 (the wide tile of
// a family that pair_rows_supported, without a dipole term)
int narrow_tile_rows(int family);
bool pair_rows_supported(int family);
// map: the tensor map of the gathered buffer for TMA plane loads (null:
// planes staged through registers); tma_box gives its box geometry
// tz: cells along z of the tile, 32 or (simple cubic, wide rows, no dipole
// term, no TMA) the half-width 16
cudaError_t launch_tiled(int family, int tz, int ty, int rpt, int occupancy, int stage, unsigned grid,
                         cudaStream_t st, const Params& P, const TiledParams& TP, const float* s0, const float* sin,
                         float* out, float* aux, uint32_t k, uint32_t advance, bool dipole, const CUtensorMap* map);
bool tma_box(int family, int ty, int* lo, int* width, int* rows);
// fused Heun step (llg_fused.cuh, instantiated by llg_fused_a.cu and
// llg_fused_b.cu): one launch per step, s0 -> s1; tile rows fused_rows()
bool fused_supported(int family);
int fused_rows(int family, bool wide);
cudaError_t launch_fused(int family, bool wide, int occupancy, unsigned grid, cudaStream_t st, const Params& P,
                         const TiledParams& TP, const float* s0, float* s1, uint32_t k, uint32_t adv);
template <bool DIP, int RPT, bool TMA>
cudaError_t launch_tiled_t(int family, int ty, int occupancy, int stage, unsigned grid, cudaStream_t st,
                           const Params& P, const TiledParams& TP, const float* s0, const float* sin, float* out,
                           float* aux, uint32_t k, uint32_t adv, const CUtensorMap* map);

// observables (llg_observe.cu): ordered per-tile partial sums copied to
// h_partials [ntiles][nq] = (sum mu_s Sx, Sy, Sz, sum mu_s, E_term...)
int observe(const Params& P, const void* state, bool fp64, int replica, int first_tile, int ntiles,
            double* d_partials, double* h_partials, int nq, cudaStream_t stream);
int topological_charge(const Params& P, const void* state, bool fp64, int replica, int ntiles_max,
                       double* d_partials, double* h_partials, cudaStream_t stream, double* q);

}  // namespace jams_llg
