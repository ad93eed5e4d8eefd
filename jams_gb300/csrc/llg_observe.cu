// On-device FP64 observables of one replica: magnetisation, energy of every
// Hamiltonian term, topological charge.  The reference computes these on the
// host after a full device-to-host copy of the spins
// (src/jams/monitors/magnetisation.cc:77-104, src/jams/monitors/energy.cc:22-33,
// src/jams/monitors/topological_charge_geometrical_def.cc:159-181); here each
// 256-spin tile reduces in shared memory in a fixed tree order and the host
// adds the per-tile partials in tile order, so results do not depend on
// scheduling: a shuffle tree inside each warp, then the warps in order.
#include <cmath>

#include "llg_kernels.h"

namespace jams_llg {

namespace {

template <typename Real>
__device__ __forceinline__ void load3(const Real* base, int64_t npad, int64_t j, double v[3]) {
  v[0] = (double)base[j];
  v[1] = (double)base[npad + j];
  v[2] = (double)base[2 * npad + j];
}

__device__ __forceinline__ int cls_total(const ReplicaDev& R) { return R.ncls[0] * R.ncls[1] * R.ncls[2]; }

// sum over the block in a fixed order: a shuffle tree inside each warp, then
// the warps' sums in warp order by thread 0 (the only thread that gets the
// total); every thread of the block calls it
__device__ __forceinline__ double block_sum(double v, double* warp_sums) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = v;
  __syncthreads();
  double total = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < kBlock / 32; ++k) total += warp_sums[k];
  __syncthreads();
  return total;
}

__device__ __forceinline__ int axis_class_o(int c, int L, int R, int ncls) {
  if (ncls == L) return c;
  if (c < R) return c;
  if (c >= L - R) return c - (L - R) + R + 1;
  return R;
}

// per-spin contributions: q0..2 = mu_s S, q3 = mu_s, q4+t = energy of term t,
// then per basis site b: q[4 + nterms + 4b + 0..3] = mu_s S, mu_s of the
// site's spins (zero elsewhere), for the magnetisation by material or
// position (src/jams/monitors/magnetisation.cc:20-104)
template <typename Real>
__global__ void __launch_bounds__(kBlock) observe_kernel(const __grid_constant__ Params P,
                                                         const Real* __restrict__ s, int first_tile,
                                                         double* __restrict__ partials, int nq) {
  __shared__ double red[kBlock / 32];
  const int tile_index = first_tile + blockIdx.x;
  const int2 tile = P.tiles[tile_index];
  const ReplicaDev& R = P.rep[tile.x];
  const int32_t i = tile.y + (int32_t)threadIdx.x;
  const bool active = i < R.n;
  double q[4 + kMaxTerms + 4 * kMaxBasis];
#pragma unroll
  for (int k = 0; k < 4 + kMaxTerms + 4 * kMaxBasis; ++k) q[k] = 0.0;
  if (active) {
    const int64_t gi = R.offset + i;
    const int b = i % P.nb;
    const int32_t c = i / P.nb;
    const int32_t c3 = c % R.L[2];
    const int32_t tt = c / R.L[2];
    const int32_t c2 = tt % R.L[1];
    const int32_t c1 = tt / R.L[1];
    const int cl = (axis_class_o(c1, R.L[0], R.R[0], R.ncls[0]) * R.ncls[1] +
                    axis_class_o(c2, R.L[1], R.R[1], R.ncls[1])) * R.ncls[2] +
                   axis_class_o(c3, R.L[2], R.R[2], R.ncls[2]);
    double sv[3];
    load3(s, P.npad, gi, sv);
    const double mu = P.mus[b];
    q[0] = mu * sv[0];
    q[1] = mu * sv[1];
    q[2] = mu * sv[2];
    q[3] = mu;
    double* qb = q + 4 + P.nterms + 4 * b;
    qb[0] = q[0];
    qb[1] = q[1];
    qb[2] = q[2];
    qb[3] = mu;
    for (int t = 0; t < P.nterms; ++t) {
      const TermDev& T = P.term[t];
      double e = 0.0;
      if (T.kind == kExchange) {
        // -1/2 S . (sum_j J_ij S_j)   (sparse_interaction.cc:86-100)
        const int x = T.exch;
        const int64_t clsi = (int64_t)b * cls_total(R) + cl;
        const int2* list = P.tab64 + R.tab64[x] + clsi * P.zmax[x];
        const int cnt = P.cnt64[R.cnt64[x] + clsi];
        double f[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < cnt; ++k) {
          const int2 ent = list[k];
          double sj[3];
          if (!LLG_IN_RANGE(P, gi + ent.x, R.offset, R.offset + R.n)) continue;
          load3(s, P.npad, gi + ent.x, sj);
          const double* J = P.ex64[x].J + (int64_t)ent.y * 9;
          for (int m = 0; m < 3; ++m) f[m] += J[3 * m] * sj[0] + J[3 * m + 1] * sj[1] + J[3 * m + 2] * sj[2];
        }
        e = -0.5 * (sv[0] * f[0] + sv[1] * f[1] + sv[2] * f[2]);
      } else if (T.kind == kUniaxial) {
        // -K (S.a)^p   (uniaxial_anisotropy.cc:126-133)
        const double* a = T.axis[b];
        const double d = a[0] * sv[0] + a[1] * sv[1] + a[2] * sv[2];
        double p = d * d;
        if (T.order >= 4) p = p * d * d;
        if (T.order >= 6) p = p * d * d;
        e = -T.K[b] * p;
      } else if (T.kind == kCubic) {
        // (cubic_anisotropy.cc:135-156)
        const double* u = T.axis[b];
        const double Su = u[0] * sv[0] + u[1] * sv[1] + u[2] * sv[2];
        const double Sv = u[3] * sv[0] + u[4] * sv[1] + u[5] * sv[2];
        const double Sw = u[6] * sv[0] + u[7] * sv[1] + u[8] * sv[2];
        const double Su2 = Su * Su, Sv2 = Sv * Sv, Sw2 = Sw * Sw;
        e = T.order == 1 ? -T.K[b] * (Su2 * Sv2 + Sv2 * Sw2 + Sw2 * Su2) : -T.K[b] * (Su2 * Sv2 * Sw2);
      } else if (T.kind == kDipole) {
        // -1/2 S . h_dip   (cuda_dipole_fft.cu:156-167); planes computed for s
        const Real* hd = dipole_planes<Real>(P);
        if (hd)
          e = -0.5 * (sv[0] * (double)hd[gi] + sv[1] * (double)hd[P.npad + gi] +
                      sv[2] * (double)hd[2 * P.npad + gi]);
      } else if (T.kind == kZeeman) {
        // -S . (mu_s B_dc + mu_s B_ac cos(w t)) at the solver time (zeeman.cc:82-87)
        const double* pf = P.pulse_now64;
        double f[3];
        for (int m = 0; m < 3; ++m) f[m] = (T.order && pf) ? T.axis[b][m] + T.axis[b][3 + m] * pf[2 + b] : T.axis[b][m];
        e = -(sv[0] * f[0] + sv[1] * f[1] + sv[2] * f[2]);
      } else {
        // -S . (mu_s B f(t)) at the solver time   (applied_field.cc:150-155)
        const double* pf = P.pulse_now64;
        double f[3];
        for (int m = 0; m < 3; ++m) f[m] = mu * (pf ? (R.B[m] * pf[0]) * pf[1] : R.B[m]);
        e = -(sv[0] * f[0] + sv[1] * f[1] + sv[2] * f[2]);
      }
      q[4 + t] = e;
    }
  }
  for (int k = 0; k < nq; ++k) {
    const double total = block_sum(q[k], red);
    if (threadIdx.x == 0) partials[(int64_t)blockIdx.x * nq + k] = total;
  }
}

__device__ __forceinline__ double solid_angle(const double* a, const double* b, const double* c) {
  const double bxc[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]};
  const double triple = a[0] * bxc[0] + a[1] * bxc[1] + a[2] * bxc[2];
  const double ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
  const double ac = a[0] * c[0] + a[1] * c[1] + a[2] * c[2];
  const double bc = b[0] * c[0] + b[1] * c[1] + b[2] * c[2];
  return 2.0 * atan2(triple, 1.0 + ab + ac + bc);
}

// one thread per cell of a one-site triangular monolayer: triangles
// (c, c + a1, c + a2) and (c + a1, c + a1 + a2, c + a2), counter-clockwise
template <typename Real>
__global__ void __launch_bounds__(kBlock) charge_kernel(const __grid_constant__ Params P, const Real* __restrict__ s,
                                                        int replica, double* __restrict__ partials) {
  __shared__ double red[kBlock / 32];
  const ReplicaDev& R = P.rep[replica];
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  const int L1 = R.L[0], L2 = R.L[1];
  double qsum = 0.0;
  if (i < (int64_t)L1 * L2) {
    const int c1 = (int)(i / L2), c2 = (int)(i % L2);
    const int p1 = c1 + 1 == L1 ? 0 : c1 + 1;
    const int p2 = c2 + 1 == L2 ? 0 : c2 + 1;
    double s00[3], s10[3], s01[3], s11[3];
    load3(s, P.npad, R.offset + (int64_t)c1 * L2 + c2, s00);
    load3(s, P.npad, R.offset + (int64_t)p1 * L2 + c2, s10);
    load3(s, P.npad, R.offset + (int64_t)c1 * L2 + p2, s01);
    load3(s, P.npad, R.offset + (int64_t)p1 * L2 + p2, s11);
    qsum = solid_angle(s00, s10, s01) + solid_angle(s10, s11, s01);
  }
  const double total = block_sum(qsum, red);
  if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

}  // namespace

int observe(const Params& P, const void* state, bool fp64, int replica, int first_tile, int ntiles,
            double* d_partials, double* h_partials, int nq, cudaStream_t stream) {
  (void)replica;
  if (fp64)
    observe_kernel<double><<<ntiles, kBlock, 0, stream>>>(P, (const double*)state, first_tile, d_partials, nq);
  else
    observe_kernel<float><<<ntiles, kBlock, 0, stream>>>(P, (const float*)state, first_tile, d_partials, nq);
  if (cudaGetLastError() != cudaSuccess) return -1;
  if (cudaMemcpyAsync(h_partials, d_partials, sizeof(double) * (size_t)ntiles * nq, cudaMemcpyDeviceToHost,
                      stream) != cudaSuccess)
    return -1;
  return cudaStreamSynchronize(stream) == cudaSuccess ? 0 : -1;
}

int topological_charge(const Params& P, const void* state, bool fp64, int replica, int ntiles_max,
                       double* d_partials, double* h_partials, cudaStream_t stream, double* q) {
  ReplicaDev R;
  if (cudaMemcpy(&R, P.rep + replica, sizeof R, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  const int64_t cells = (int64_t)R.L[0] * R.L[1];
  const int nblk = (int)((cells + kBlock - 1) / kBlock);
  if (nblk > ntiles_max * (4 + kMaxTerms)) return -1;
  if (fp64)
    charge_kernel<double><<<nblk, kBlock, 0, stream>>>(P, (const double*)state, replica, d_partials);
  else
    charge_kernel<float><<<nblk, kBlock, 0, stream>>>(P, (const float*)state, replica, d_partials);
  if (cudaGetLastError() != cudaSuccess) return -1;
  if (cudaMemcpyAsync(h_partials, d_partials, sizeof(double) * nblk, cudaMemcpyDeviceToHost, stream) !=
      cudaSuccess)
    return -1;
  if (cudaStreamSynchronize(stream) != cudaSuccess) return -1;
  double sum = 0.0;
  for (int k = 0; k < nblk; ++k) sum += h_partials[k];
  *q = sum / (4.0 * 3.14159265358979323846264338327950288);
  return 0;
}

}  // namespace jams_llg
