// Fused stochastic-LLG stage kernels for sm_103a.
//
// One launch = one integrator stage over every spin of every replica: the
// effective field of all Hamiltonian terms, the in-kernel thermal noise and
// the LLG update are evaluated in registers and only spin vectors cross HBM.
// This replaces, per stage, the reference's cusparseSpMV + per-term kernels +
// cudaMemcpy/cublasDaxpy summation + cuRAND + integrator kernels
// (src/jams/solvers/cuda_llg_heun.cu:64-122, src/jams/cuda/cuda_solver.cc:11-26).
//
// Two arithmetic forms:
//   FP64 ("plain"): every operation is an explicitly rounded __dmul_rn /
//     __dadd_rn / __ddiv_rn / __dsqrt_rn in the association order of the
//     reference's CPU code (no FMA contraction), and the neighbours of each
//     spin are visited in ascending site index as the CSR row sum of
//     Xcsrmv_general does (src/jams/interface/sparse_blas.h:13-27).  The
//     result equals the CPU solver's bit for bit.
//   FP32C: FP32 spins and fields; isotropic exchange summed per shell and
//     the shells combined with error-free transformations (TwoProd by FMA,
//     TwoSum), i.e. a compensated neighbour sum; FP64 noise prefactors.
//
// Thread mapping: one thread per spin, 256-spin tiles of one replica per
// CTA (the replica work-list), neighbours gathered through L1 from the SoA
// planes (32 consecutive spins of a warp read 32 consecutive floats per
// neighbour slot: coalesced 128-byte lines).
#include <cfloat>
#include <cstdint>

#include "llg_kernels.h"
#include "llg_noise.cuh"

namespace jams_llg {

// ---------------------------------------------------------------- helpers --

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dd(double a, double b) { return __ddiv_rn(a, b); }

template <typename Real>
struct Planes {
  Real* x;
  Real* y;
  Real* z;
};

template <typename Real>
__device__ __forceinline__ Planes<Real> planes(Real* base, int64_t npad) {
  return Planes<Real>{base, base + npad, base + 2 * npad};
}

struct Site {
  int32_t b;
  int32_t q;   // boundary class
};

__device__ __forceinline__ int axis_class(int c, int L, int R, int ncls) {
  if (ncls == L) return c;
  if (c < R) return c;
  if (c >= L - R) return c - (L - R) + R + 1;
  return R;
}

__device__ __forceinline__ Site locate(const ReplicaDev& R, int nb, int32_t i) {
  Site s;
  s.b = i % nb;
  const int32_t c = i / nb;
  const int32_t c3 = c % R.L[2];
  const int32_t t = c / R.L[2];
  const int32_t c2 = t % R.L[1];
  const int32_t c1 = t / R.L[1];
  const int k1 = axis_class(c1, R.L[0], R.R[0], R.ncls[0]);
  const int k2 = axis_class(c2, R.L[1], R.R[1], R.ncls[1]);
  const int k3 = axis_class(c3, R.L[2], R.R[2], R.ncls[2]);
  s.q = (k1 * R.ncls[1] + k2) * R.ncls[2] + k3;
  return s;
}

__device__ __forceinline__ int nclass_total(const ReplicaDev& R) {
  return R.ncls[0] * R.ncls[1] * R.ncls[2];
}

// error-free transformations (Knuth TwoSum; TwoProd by FMA)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// h (hi, lo) += c, compensated
__device__ __forceinline__ void acc_add(float& hi, float& lo, float c) {
  float s, e;
  two_sum(hi, c, s, e);
  hi = s;
  lo = __fadd_rn(lo, e);
}

// h (hi, lo) += (jhi + jlo) * a, compensated
__device__ __forceinline__ void acc_mad(float& hi, float& lo, float jhi, float jlo, float a) {
  const float p = __fmul_rn(jhi, a);
  const float pe = __fmaf_rn(jhi, a, -p);
  float s, e;
  two_sum(hi, p, s, e);
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(e, __fmaf_rn(jlo, a, pe)));
}

// ------------------------------------------------------------ FP32 fields --

// exchange term t, compensated; spins read from planes S
__device__ __forceinline__ void exchange_f32(const Params& P, int t, const ReplicaDev& R, Site st,
                                             int64_t gi, const Planes<const float>& S, float hi[3],
                                             float lo[3]) {
  const ExchangeF32& E = P.ex32[t];
  const int b = st.b;
  const int32_t* tab = P.tab32 + R.tab32[t] +
                       ((int64_t)b * nclass_total(R) + st.q) * P.nslot_max[t];
  int slot = 0;
  const int ng = E.ngroup[b];
  for (int g = 0; g < ng; ++g) {
    float ax = 0.f, ay = 0.f, az = 0.f;
    const int end = E.group_end[b][g];
    for (; slot < end; ++slot) {
      const int32_t off = __ldg(tab + slot);
      if (off != kMissing && LLG_IN_RANGE(P, gi + off, R.offset, R.offset + R.n)) {
        const int64_t j = gi + off;
        ax += __ldg(S.x + j);
        ay += __ldg(S.y + j);
        az += __ldg(S.z + j);
      }
    }
    const float jh = E.group_j_hi[b][g], jl = E.group_j_lo[b][g];
    acc_mad(hi[0], lo[0], jh, jl, ax);
    acc_mad(hi[1], lo[1], jh, jl, ay);
    acc_mad(hi[2], lo[2], jh, jl, az);
  }
  const int ns = E.nslot[b];
  for (; slot < ns; ++slot) {
    const int32_t off = __ldg(tab + slot);
    if (off == kMissing || !LLG_IN_RANGE(P, gi + off, R.offset, R.offset + R.n)) continue;
    const int64_t j = gi + off;
    const float sx = __ldg(S.x + j), sy = __ldg(S.y + j), sz = __ldg(S.z + j);
    const float* Jr = E.rest_j + ((int64_t)b * kMaxSlots + slot) * 9;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const float c = __fmaf_rn(__ldg(Jr + 3 * m + 2), sz,
                                __fmaf_rn(__ldg(Jr + 3 * m + 1), sy, __fmul_rn(__ldg(Jr + 3 * m), sx)));
      acc_add(hi[m], lo[m], c);
    }
  }
}

// total field (meV) of all terms at spin s, compensated, FP32; pf: the time
// factors of the stage (null: no time-dependent field); only >= 0: the field
// of that term alone
__device__ __forceinline__ void field_f32(const Params& P, const ReplicaDev& R, Site st, int64_t gi,
                                          const Planes<const float>& S, const float s[3], float h[3],
                                          const float* hd, const float* pf, int only = -1) {
  float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
  const int b = st.b;
  for (int t = 0; t < P.nterms; ++t) {
    if (only >= 0 && t != only) continue;
    const TermDev& T = P.term[t];
    switch (T.kind) {
      case kExchange:
        exchange_f32(P, T.exch, R, st, gi, S, hi, lo);
        break;
      case kUniaxial: {
        const float* a = T.axisf[b];
        const float d = __fmaf_rn(a[2], s[2], __fmaf_rn(a[1], s[1], a[0] * s[0]));
        float pw = d;  // d^(p-1)
        if (T.order >= 4) pw = d * d * d;
        if (T.order >= 6) pw = pw * d * d;
        const float pre = T.Kf[b] * (float)T.order * pw;
#pragma unroll
        for (int m = 0; m < 3; ++m) acc_add(hi[m], lo[m], pre * a[m]);
        break;
      }
      case kCubic: {
        const float* u = T.axisf[b];
        const float* v = u + 3;
        const float* w = u + 6;
        const float Su = u[0] * s[0] + u[1] * s[1] + u[2] * s[2];
        const float Sv = v[0] * s[0] + v[1] * s[1] + v[2] * s[2];
        const float Sw = w[0] * s[0] + w[1] * s[1] + w[2] * s[2];
        const float pre = 2.0f * T.Kf[b];
        float cu, cv, cw;
        if (T.order == 1) {
          cu = Su * (Sv * Sv + Sw * Sw);
          cv = Sv * (Sw * Sw + Su * Su);
          cw = Sw * (Su * Su + Sv * Sv);
        } else {
          cu = Su * (Sv * Sv) * (Sw * Sw);
          cv = Sv * (Sw * Sw) * (Su * Su);
          cw = Sw * (Su * Su) * (Sv * Sv);
        }
#pragma unroll
        for (int m = 0; m < 3; ++m) acc_add(hi[m], lo[m], pre * (u[m] * cu + v[m] * cv + w[m] * cw));
        break;
      }
      case kDipole:  // precomputed by FFT convolution for these spins
        if (hd) {
#pragma unroll
          for (int m = 0; m < 3; ++m) acc_add(hi[m], lo[m], hd[m * P.npad + gi]);
        }
        break;
      case kZeeman: {  // mu_s B_dc + mu_s B_ac cos(w t)
#pragma unroll
        for (int m = 0; m < 3; ++m)
          acc_add(hi[m], lo[m], T.order ? T.axisf[b][m] + T.axisf[b][3 + m] * pf[2 + b] : T.axisf[b][m]);
        break;
      }
      default: {  // applied field: mu_s B, times the pulse factors
#pragma unroll
        for (int m = 0; m < 3; ++m) acc_add(hi[m], lo[m], P.mus32[b] * (pf ? R.Bf[m] * pf[0] * pf[1] : R.Bf[m]));
        break;
      }
    }
  }
#pragma unroll
  for (int m = 0; m < 3; ++m) h[m] = hi[m] + lo[m];
}

// LLG right-hand side from the total field h (meV), FP32:
// rhs = -gamma (S x H' + alpha S x (S x H')), H' = h / mu_s + xi
__device__ __forceinline__ void rhs_f32(const Params& P, int b, const float s[3], const float h[3],
                                        const float w[3], float rhs[3]) {
  const float im = P.inv_mus32[b];
  const float hh[3] = {__fmaf_rn(h[0], im, w[0]), __fmaf_rn(h[1], im, w[1]), __fmaf_rn(h[2], im, w[2])};
  const float c1[3] = {s[1] * hh[2] - s[2] * hh[1], s[2] * hh[0] - s[0] * hh[2], s[0] * hh[1] - s[1] * hh[0]};
  const float c2[3] = {s[1] * c1[2] - s[2] * c1[1], s[2] * c1[0] - s[0] * c1[2], s[0] * c1[1] - s[1] * c1[0]};
  const float mg = -P.gyro32[b], a = P.alpha32[b];
#pragma unroll
  for (int m = 0; m < 3; ++m) rhs[m] = mg * __fmaf_rn(a, c2[m], c1[m]);
}

__device__ __forceinline__ void noise_f32(const Params& P, const ReplicaDev& R, int r, int b, int32_t i,
                                          uint64_t step, float w[3]) {
  if (R.thermal) {
    float z[3];
    noise_normals(P.seed, (uint32_t)r, step, (uint32_t)i, z);
    const float amp = R.amp32[b];
    w[0] = z[0] * amp;
    w[1] = z[1] * amp;
    w[2] = z[2] * amp;
  } else {
    w[0] = w[1] = w[2] = 0.f;
  }
}

__device__ __forceinline__ void normalise_f32(float v[3]) {
  const float r = rsqrtf(__fmaf_rn(v[2], v[2], __fmaf_rn(v[1], v[1], v[0] * v[0])));
  v[0] *= r;
  v[1] *= r;
  v[2] *= r;
}

__device__ __forceinline__ void flag_nonfinite(const Params& P, const float v[3]) {
  if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) atomicOr(P.status, 1u);
}

// ------------------------------------------------------------ FP64 fields --

// exchange term t in ascending neighbour order, CSR association:
// sum_m = ((0 + s_j0[n] J0[m][n]) + s_j1[n] J1[m][n]) + ...
__device__ __forceinline__ void exchange_f64(const Params& P, int t, const ReplicaDev& R, Site st,
                                             int64_t gi, const Planes<const double>& S, double f[3]) {
  const ExchangeF64& E = P.ex64[t];
  const int64_t cls = (int64_t)st.b * nclass_total(R) + st.q;
  const int2* list = P.tab64 + R.tab64[t] + cls * P.zmax[t];
  const int cnt = __ldg(P.cnt64 + R.cnt64[t] + cls);
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int k = 0; k < cnt; ++k) {
    const int2 ent = __ldg(list + k);
    const int64_t j = gi + ent.x;
    if (!LLG_IN_RANGE(P, j, R.offset, R.offset + R.n)) continue;
    const double sj[3] = {__ldg(S.x + j), __ldg(S.y + j), __ldg(S.z + j)};
    const double* J = E.J + (int64_t)ent.y * 9;
    const unsigned mask = __ldg(E.mask + ent.y);
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      if (mask & (1u << n)) s0 = da(s0, dm(sj[n], __ldg(J + n)));
    }
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      if (mask & (1u << (3 + n))) s1 = da(s1, dm(sj[n], __ldg(J + 3 + n)));
    }
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      if (mask & (1u << (6 + n))) s2 = da(s2, dm(sj[n], __ldg(J + 6 + n)));
    }
  }
  f[0] = s0;
  f[1] = s1;
  f[2] = s2;
}

// one term's field, FP64, reference association order; pf: the time factors
// of the stage (null: no time-dependent field)
__device__ __forceinline__ void term_field_f64(const Params& P, const TermDev& T, const ReplicaDev& R,
                                               Site st, int64_t gi, const Planes<const double>& S,
                                               const double s[3], double f[3], const double* hd,
                                               const double* pf) {
  const int b = st.b;
  switch (T.kind) {
    case kExchange:
      exchange_f64(P, T.exch, R, st, gi, S, f);
      break;
    case kUniaxial: {
      // src/jams/hamiltonian/uniaxial_anisotropy.cc:155-163
      const double* a = T.axis[b];
      const double d = da(da(dm(a[0], s[0]), dm(a[1], s[1])), dm(a[2], s[2]));
      double pw = d;
      if (T.order >= 4) pw = dm(dm(d, d), d);
      if (T.order >= 6) pw = dm(dm(pw, d), d);
      const double pre = dm(dm(T.K[b], (double)T.order), pw);
#pragma unroll
      for (int m = 0; m < 3; ++m) f[m] = dm(pre, a[m]);
      break;
    }
    case kCubic: {
      // src/jams/hamiltonian/cubic_anisotropy.cc:197-226
      const double* u = T.axis[b];
      const double* v = u + 3;
      const double* w = u + 6;
      const double Su = da(da(dm(s[0], u[0]), dm(s[1], u[1])), dm(s[2], u[2]));
      const double Sv = da(da(dm(s[0], v[0]), dm(s[1], v[1])), dm(s[2], v[2]));
      const double Sw = da(da(dm(s[0], w[0]), dm(s[1], w[1])), dm(s[2], w[2]));
      const double Su2 = dm(Su, Su), Sv2 = dm(Sv, Sv), Sw2 = dm(Sw, Sw);
      const double pre = dm(2.0, T.K[b]);
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        double x;
        if (T.order == 1) {
          x = da(da(dm(dm(u[m], Su), da(Sv2, Sw2)), dm(dm(v[m], Sv), da(Sw2, Su2))),
                 dm(dm(w[m], Sw), da(Su2, Sv2)));
        } else {
          x = da(da(dm(dm(dm(u[m], Su), Sv2), Sw2), dm(dm(dm(v[m], Sv), Sw2), Su2)),
                 dm(dm(dm(w[m], Sw), Su2), Sv2));
        }
        f[m] = da(0.0, dm(pre, x));
      }
      break;
    }
    case kDipole:
      // precomputed by FFT convolution (cuda_dipole_fft.cu:184-209)
#pragma unroll
      for (int m = 0; m < 3; ++m) f[m] = hd ? hd[m * P.npad + gi] : 0.0;
      break;
    case kZeeman:
      // dc_local_field + ac_local_field cos(w t), both already times mu_s
      // (src/jams/hamiltonian/zeeman.cc:26-71,106-121)
#pragma unroll
      for (int m = 0; m < 3; ++m) f[m] = T.order ? da(T.axis[b][m], dm(T.axis[b][3 + m], pf[2 + b])) : T.axis[b][m];
      break;
    default: {
      // mu_s (B sinc) cos (src/jams/hamiltonian/applied_field.cc:17-78,
      // 146-148); static: mu_s B
#pragma unroll
      for (int m = 0; m < 3; ++m) f[m] = dm(P.mus[b], pf ? dm(dm(R.B[m], pf[0]), pf[1]) : R.B[m]);
      break;
    }
  }
}

// Solver::compute_fields: copy of term 0 then daxpy(1.0) of the others
__device__ __forceinline__ void field_f64(const Params& P, const ReplicaDev& R, Site st, int64_t gi,
                                          const Planes<const double>& S, const double s[3], double h[3],
                                          const double* hd, const double* pf) {
  h[0] = h[1] = h[2] = 0.0;
  for (int t = 0; t < P.nterms; ++t) {
    double f[3];
    term_field_f64(P, P.term[t], R, st, gi, S, s, f, hd, pf);
    if (t == 0) {
      h[0] = f[0];
      h[1] = f[1];
      h[2] = f[2];
    } else {
      h[0] = da(h[0], dm(1.0, f[0]));
      h[1] = da(h[1], dm(1.0, f[1]));
      h[2] = da(h[2], dm(1.0, f[2]));
    }
  }
}

// H' = w + h / mu_s (T > 0) or h / mu_s; rhs = -g (S x H' + a S x (S x H'))
__device__ __forceinline__ void rhs_f64(const Params& P, int b, bool thermal, const double s[3],
                                        const double h[3], const double w[3], double rhs[3]) {
  double hh[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) hh[m] = thermal ? da(w[m], dd(h[m], P.mus[b])) : dd(h[m], P.mus[b]);
  const double c1[3] = {dsub(dm(s[1], hh[2]), dm(s[2], hh[1])), dsub(dm(s[2], hh[0]), dm(s[0], hh[2])),
                        dsub(dm(s[0], hh[1]), dm(s[1], hh[0]))};
  const double c2[3] = {dsub(dm(s[1], c1[2]), dm(s[2], c1[1])), dsub(dm(s[2], c1[0]), dm(s[0], c1[2])),
                        dsub(dm(s[0], c1[1]), dm(s[1], c1[0]))};
  const double mg = -P.gyro[b], a = P.alpha[b];
#pragma unroll
  for (int m = 0; m < 3; ++m) rhs[m] = dm(mg, da(c1[m], dm(a, c2[m])));
}

__device__ __forceinline__ void noise_f64(const Params& P, const ReplicaDev& R, int r, int b, int32_t i,
                                          uint64_t step, double w[3]) {
  if (R.thermal) {
    float z[3];
    noise_normals(P.seed, (uint32_t)r, step, (uint32_t)i, z);
#pragma unroll
    for (int m = 0; m < 3; ++m) w[m] = dm(dm((double)z[m], P.sigma[b]), R.sqrt_t);
  } else {
    w[0] = w[1] = w[2] = 0.0;
  }
}

// unit_vector (src/jams/containers/vec3.h:275-283)
__device__ __forceinline__ void unit_vector_f64(double v[3]) {
  const double len = __dsqrt_rn(da(da(dm(v[0], v[0]), dm(v[1], v[1])), dm(v[2], v[2])));
  if (fabs(len) <= DBL_EPSILON) return;
  v[0] = dd(v[0], len);
  v[1] = dd(v[1], len);
  v[2] = dd(v[2], len);
}

__device__ __forceinline__ void flag_nonfinite(const Params& P, const double v[3]) {
  if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) atomicOr(P.status, 1u);
}

// ----------------------------------------------------------------- tiles --

struct Me {
  int r;
  int32_t i;
  int64_t gi;
  bool active;
};

__device__ __forceinline__ Me whoami(const Params& P, const ReplicaDev*& Rp) {
  const int2 tile = __ldg(P.tiles + blockIdx.x);
  Me me;
  me.r = tile.x;
  Rp = P.rep + tile.x;
  me.i = tile.y + (int32_t)threadIdx.x;
  me.active = me.i < Rp->n;
  me.gi = Rp->offset + me.i;
  return me;
}

// ================================================================== Heun ==

// predictor: s_pred = unit(s0 + dt rhs(s0)); FP64 also stores ds = rhs/2
// rhs0 (non-null): the corrector's partial sum s0 + dt/2 rhs(s0) stored
__global__ void __launch_bounds__(kBlock) heun_predict_f32(const __grid_constant__ Params P, const float* __restrict__ s0,
                                                          float* __restrict__ sp, float* __restrict__ rhs0,
                                                          uint32_t kstep) {
  const ReplicaDev* Rp;
  const Me me = whoami(P, Rp);
  if (!me.active) return;
  const ReplicaDev& R = *Rp;
  const uint64_t step = *P.step_base + kstep;
  const Site st = locate(R, P.nb, me.i);
  const Planes<const float> S = planes(s0, P.npad);
  const float s[3] = {S.x[me.gi], S.y[me.gi], S.z[me.gi]};
  float h[3], w[3], rhs[3];
  field_f32(P, R, st, me.gi, S, s, h, P.hdip32, pulse_at32(P, step, 0));
  noise_f32(P, R, me.r, st.b, me.i, step, w);
  rhs_f32(P, st.b, s, h, w, rhs);
  float v[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) v[m] = __fmaf_rn(P.dt32, rhs[m], s[m]);
  normalise_f32(v);
  const Planes<float> O = planes(sp, P.npad);
  O.x[me.gi] = v[0];
  O.y[me.gi] = v[1];
  O.z[me.gi] = v[2];
  if (rhs0) {
    const float hdt = 0.5f * P.dt32;
    const Planes<float> A = planes(rhs0, P.npad);
    A.x[me.gi] = __fmaf_rn(hdt, rhs[0], s[0]);
    A.y[me.gi] = __fmaf_rn(hdt, rhs[1], s[1]);
    A.z[me.gi] = __fmaf_rn(hdt, rhs[2], s[2]);
  }
}

// corrector: s1 = unit(a + dt/2 rhs(s_pred)) with a = s0 + dt/2 rhs(s0),
// read from the predictor's store (rhs0 non-null, the same value) or
// recomputed
__global__ void __launch_bounds__(kBlock) heun_correct_f32(const __grid_constant__ Params P, const float* __restrict__ s0,
                                                          const float* __restrict__ sp, float* __restrict__ s1,
                                                          const float* __restrict__ rhs0, uint32_t kstep) {
  const ReplicaDev* Rp;
  const Me me = whoami(P, Rp);
  if (!me.active) return;
  const ReplicaDev& R = *Rp;
  const uint64_t step = *P.step_base + kstep;
  const Site st = locate(R, P.nb, me.i);
  const Planes<const float> SP = planes(sp, P.npad);
  const float p[3] = {SP.x[me.gi], SP.y[me.gi], SP.z[me.gi]};
  const float hdt = 0.5f * P.dt32;
  float w[3];
  noise_f32(P, R, me.r, st.b, me.i, step, w);
  float h[3], a[3], r1[3];
  if (rhs0) {
    const Planes<const float> A = planes(rhs0, P.npad);
    a[0] = A.x[me.gi];
    a[1] = A.y[me.gi];
    a[2] = A.z[me.gi];
  }
  field_f32(P, R, st, me.gi, SP, p, h, P.hdip32, pulse_at32(P, step, 1));
  rhs_f32(P, st.b, p, h, w, r1);
  if (!rhs0) {
    const Planes<const float> S0 = planes(s0, P.npad);
    const float q[3] = {S0.x[me.gi], S0.y[me.gi], S0.z[me.gi]};
    float r0[3];
    field_f32(P, R, st, me.gi, S0, q, h, P.hdip32_s0, pulse_at32(P, step, 0));
    rhs_f32(P, st.b, q, h, w, r0);
#pragma unroll
    for (int m = 0; m < 3; ++m) a[m] = __fmaf_rn(hdt, r0[m], q[m]);
  }
  float v[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) v[m] = __fmaf_rn(hdt, r1[m], a[m]);
  normalise_f32(v);
  flag_nonfinite(P, v);
  const Planes<float> O = planes(s1, P.npad);
  O.x[me.gi] = v[0];
  O.y[me.gi] = v[1];
  O.z[me.gi] = v[2];
}

// FP64: src/jams/solvers/cpu_llg_heun.cc:84-102
__global__ void __launch_bounds__(kBlock) heun_predict_f64(const __grid_constant__ Params P, const double* __restrict__ s0,
                                                          double* __restrict__ sp, double* __restrict__ ds,
                                                          uint32_t kstep) {
  const ReplicaDev* Rp;
  const Me me = whoami(P, Rp);
  if (!me.active) return;
  const ReplicaDev& R = *Rp;
  const uint64_t step = *P.step_base + kstep;
  const Site st = locate(R, P.nb, me.i);
  const Planes<const double> S = planes(s0, P.npad);
  const double s[3] = {S.x[me.gi], S.y[me.gi], S.z[me.gi]};
  double h[3], w[3], rhs[3];
  field_f64(P, R, st, me.gi, S, s, h, P.hdip64, pulse_at64(P, step, 0));
  noise_f64(P, R, me.r, st.b, me.i, step, w);
  rhs_f64(P, st.b, R.thermal != 0, s, h, w, rhs);
  const Planes<double> D = planes(ds, P.npad);
  double v[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) v[m] = da(s[m], dm(P.dt, rhs[m]));
  D.x[me.gi] = dm(0.5, rhs[0]);
  D.y[me.gi] = dm(0.5, rhs[1]);
  D.z[me.gi] = dm(0.5, rhs[2]);
  unit_vector_f64(v);
  const Planes<double> O = planes(sp, P.npad);
  O.x[me.gi] = v[0];
  O.y[me.gi] = v[1];
  O.z[me.gi] = v[2];
}

// FP64: src/jams/solvers/cpu_llg_heun.cc:106-145
__global__ void __launch_bounds__(kBlock) heun_correct_f64(const __grid_constant__ Params P, const double* s0,
                                                          const double* sp, const double* ds,
                                                          double* s1, uint32_t kstep) {
  const ReplicaDev* Rp;
  const Me me = whoami(P, Rp);
  if (!me.active) return;
  const ReplicaDev& R = *Rp;
  const uint64_t step = *P.step_base + kstep;
  const Site st = locate(R, P.nb, me.i);
  const Planes<const double> SP = planes(sp, P.npad);
  const double p[3] = {SP.x[me.gi], SP.y[me.gi], SP.z[me.gi]};
  double h[3], w[3], rhs[3];
  field_f64(P, R, st, me.gi, SP, p, h, P.hdip64, pulse_at64(P, step, 1));
  noise_f64(P, R, me.r, st.b, me.i, step, w);
  rhs_f64(P, st.b, R.thermal != 0, p, h, w, rhs);
  const Planes<const double> S0 = planes(s0, P.npad);
  const Planes<const double> D = planes(ds, P.npad);
  const double dsv[3] = {D.x[me.gi], D.y[me.gi], D.z[me.gi]};
  const double a[3] = {S0.x[me.gi], S0.y[me.gi], S0.z[me.gi]};
  double v[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) v[m] = da(a[m], dm(P.dt, da(dsv[m], dm(0.5, rhs[m]))));
  unit_vector_f64(v);
  flag_nonfinite(P, v);
  const Planes<double> O = planes(s1, P.npad);
  O.x[me.gi] = v[0];
  O.y[me.gi] = v[1];
  O.z[me.gi] = v[2];
}

// =================================================================== RK4 ==
// Stage k evaluates k_k = rhs(s_in) with the step's fixed noise and writes
// the next stage state s0 + c dt k_k; acc accumulates k1 + 2 k2 + 2 k3.
// Stage 4 writes unit(s0 + dt (acc + k4) / 6).  The reference's stage states
// are not normalised (src/jams/solvers/cuda_rk4_base.cu:66-101); FP32C can
// renormalise them (rk4_normalise_stages).

template <int STAGE>
__global__ void __launch_bounds__(kBlock) rk4_stage_f32(const __grid_constant__ Params P, const float* s0, const float* sin,
                                                       float* acc, float* sout,
                                                       uint32_t kstep) {
  const ReplicaDev* Rp;
  const Me me = whoami(P, Rp);
  if (!me.active) return;
  const ReplicaDev& R = *Rp;
  const uint64_t step = *P.step_base + kstep;
  const Site st = locate(R, P.nb, me.i);
  const Planes<const float> SI = planes(sin, P.npad);
  const float s[3] = {SI.x[me.gi], SI.y[me.gi], SI.z[me.gi]};
  float h[3], w[3], k[3];
  field_f32(P, R, st, me.gi, SI, s, h, P.hdip32, pulse_at32(P, step, STAGE - 1));
  noise_f32(P, R, me.r, st.b, me.i, step, w);
  rhs_f32(P, st.b, s, h, w, k);
  const Planes<const float> S0 = planes(s0, P.npad);
  const float a[3] = {S0.x[me.gi], S0.y[me.gi], S0.z[me.gi]};
  const Planes<float> A = planes(acc, P.npad);
  const Planes<float> O = planes(sout, P.npad);
  float v[3];
  if (STAGE == 4) {
    const float c = P.dt32 * (1.0f / 6.0f);
    const float ac[3] = {A.x[me.gi], A.y[me.gi], A.z[me.gi]};
#pragma unroll
    for (int m = 0; m < 3; ++m) v[m] = __fmaf_rn(c, ac[m] + k[m], a[m]);
    normalise_f32(v);
    flag_nonfinite(P, v);
  } else {
    const float c = STAGE == 3 ? P.dt32 : 0.5f * P.dt32;
    float ac[3];
    if (STAGE == 1) {
      ac[0] = k[0];
      ac[1] = k[1];
      ac[2] = k[2];
    } else {
      ac[0] = __fmaf_rn(2.0f, k[0], A.x[me.gi]);
      ac[1] = __fmaf_rn(2.0f, k[1], A.y[me.gi]);
      ac[2] = __fmaf_rn(2.0f, k[2], A.z[me.gi]);
    }
    A.x[me.gi] = ac[0];
    A.y[me.gi] = ac[1];
    A.z[me.gi] = ac[2];
#pragma unroll
    for (int m = 0; m < 3; ++m) v[m] = __fmaf_rn(c, k[m], a[m]);
    if (P.rk4_normalise_stages) normalise_f32(v);
  }
  O.x[me.gi] = v[0];
  O.y[me.gi] = v[1];
  O.z[me.gi] = v[2];
}

template <int STAGE>
__global__ void __launch_bounds__(kBlock) rk4_stage_f64(const __grid_constant__ Params P, const double* s0, const double* sin,
                                                       double* acc, double* sout,
                                                       uint32_t kstep) {
  const ReplicaDev* Rp;
  const Me me = whoami(P, Rp);
  if (!me.active) return;
  const ReplicaDev& R = *Rp;
  const uint64_t step = *P.step_base + kstep;
  const Site st = locate(R, P.nb, me.i);
  const Planes<const double> SI = planes(sin, P.npad);
  const double s[3] = {SI.x[me.gi], SI.y[me.gi], SI.z[me.gi]};
  double h[3], w[3], k[3];
  field_f64(P, R, st, me.gi, SI, s, h, P.hdip64, pulse_at64(P, step, STAGE - 1));
  noise_f64(P, R, me.r, st.b, me.i, step, w);
  rhs_f64(P, st.b, R.thermal != 0, s, h, w, k);
  const Planes<const double> S0 = planes(s0, P.npad);
  const double a[3] = {S0.x[me.gi], S0.y[me.gi], S0.z[me.gi]};
  const Planes<double> A = planes(acc, P.npad);
  const Planes<double> O = planes(sout, P.npad);
  double v[3];
  if (STAGE == 4) {
    // s_old + dt * (k1 + 2 k2 + 2 k3 + k4) / 6.0, then s / |s|
    const double ac[3] = {A.x[me.gi], A.y[me.gi], A.z[me.gi]};
#pragma unroll
    for (int m = 0; m < 3; ++m) v[m] = da(a[m], dd(dm(P.dt, da(ac[m], k[m])), 6.0));
    const double len = __dsqrt_rn(da(da(dm(v[0], v[0]), dm(v[1], v[1])), dm(v[2], v[2])));
    v[0] = dd(v[0], len);
    v[1] = dd(v[1], len);
    v[2] = dd(v[2], len);
    flag_nonfinite(P, v);
  } else {
    const double c = STAGE == 3 ? P.dt : dm(0.5, P.dt);
    double ac[3];
    if (STAGE == 1) {
      ac[0] = k[0];
      ac[1] = k[1];
      ac[2] = k[2];
    } else {
      ac[0] = da(A.x[me.gi], dm(2.0, k[0]));
      ac[1] = da(A.y[me.gi], dm(2.0, k[1]));
      ac[2] = da(A.z[me.gi], dm(2.0, k[2]));
    }
    A.x[me.gi] = ac[0];
    A.y[me.gi] = ac[1];
    A.z[me.gi] = ac[2];
#pragma unroll
    for (int m = 0; m < 3; ++m) v[m] = da(a[m], dm(c, k[m]));
  }
  O.x[me.gi] = v[0];
  O.y[me.gi] = v[1];
  O.z[me.gi] = v[2];
}

template __global__ void rk4_stage_f32<1>(const __grid_constant__ Params, const float*, const float*, float*, float*, uint32_t);
template __global__ void rk4_stage_f32<2>(const __grid_constant__ Params, const float*, const float*, float*, float*, uint32_t);
template __global__ void rk4_stage_f32<3>(const __grid_constant__ Params, const float*, const float*, float*, float*, uint32_t);
template __global__ void rk4_stage_f32<4>(const __grid_constant__ Params, const float*, const float*, float*, float*, uint32_t);
template __global__ void rk4_stage_f64<1>(const __grid_constant__ Params, const double*, const double*, double*, double*, uint32_t);
template __global__ void rk4_stage_f64<2>(const __grid_constant__ Params, const double*, const double*, double*, double*, uint32_t);
template __global__ void rk4_stage_f64<3>(const __grid_constant__ Params, const double*, const double*, double*, double*, uint32_t);
template __global__ void rk4_stage_f64<4>(const __grid_constant__ Params, const double*, const double*, double*, double*, uint32_t);

// ============================================================ utilities ==

// advances the noise counter base after a block of steps
__global__ void advance_step_base(uint64_t* base, uint32_t nsteps) { *base += nsteps; }

// AoS FP64 (host layout) <-> SoA planes
template <typename Real>
__global__ void unpack_state(const double* __restrict__ aos, Real* __restrict__ soa, int64_t offset,
                             int64_t n, int64_t npad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  soa[offset + i] = (Real)aos[3 * i];
  soa[npad + offset + i] = (Real)aos[3 * i + 1];
  soa[2 * npad + offset + i] = (Real)aos[3 * i + 2];
}

// SoA planes -> AoS doubles for 256 spins per block, staged through shared
// memory so that each warp writes 512 contiguous bytes (16-byte words when
// the destination is 16-byte aligned): whole cache lines, which matters most
// when the destination is mapped host memory across the host link
template <typename Real>
__global__ void __launch_bounds__(256) pack_state(const Real* __restrict__ soa, double* __restrict__ aos,
                                                  int64_t offset, int64_t n, int64_t npad) {
  __shared__ __align__(16) double buf[3 * 256];
  const int64_t base = (int64_t)blockIdx.x * 256;
  const int cnt = (int)min((int64_t)256, n - base);
  const int t = threadIdx.x;
  if (t < cnt) {
    const int64_t i = offset + base + t;
    buf[3 * t] = (double)soa[i];
    buf[3 * t + 1] = (double)soa[npad + i];
    buf[3 * t + 2] = (double)soa[2 * npad + i];
  }
  __syncthreads();
  double* out = aos + 3 * base;   // 6144-byte steps: every block has the alignment of aos
  const int words = 3 * cnt;
  if ((reinterpret_cast<uintptr_t>(out) & 15u) == 0) {
    double2* o2 = reinterpret_cast<double2*>(out);
    const double2* b2 = reinterpret_cast<const double2*>(buf);
    for (int k = t; k < words / 2; k += 256) o2[k] = b2[k];
    if ((words & 1) && t == 0) out[words - 1] = buf[words - 1];
  } else {
    for (int k = t; k < words; k += 256) out[k] = buf[k];
  }
}

template __global__ void unpack_state<float>(const double*, float*, int64_t, int64_t, int64_t);
template __global__ void unpack_state<double>(const double*, double*, int64_t, int64_t, int64_t);
template __global__ void pack_state<float>(const float*, double*, int64_t, int64_t, int64_t);
template __global__ void pack_state<double>(const double*, double*, int64_t, int64_t, int64_t);

// total field (meV) of one replica, AoS FP64 output
__global__ void __launch_bounds__(kBlock) fields_f32(const __grid_constant__ Params P, const float* __restrict__ s0,
                                                    double* __restrict__ out, int replica) {
  const ReplicaDev* Rp;
  const Me me = whoami(P, Rp);
  if (!me.active || me.r != replica) return;
  const ReplicaDev& R = *Rp;
  const Site st = locate(R, P.nb, me.i);
  const Planes<const float> S = planes(s0, P.npad);
  const float s[3] = {S.x[me.gi], S.y[me.gi], S.z[me.gi]};
  float h[3];
  field_f32(P, R, st, me.gi, S, s, h, P.hdip32, P.pulse_now32);
  out[3 * (int64_t)me.i] = h[0];
  out[3 * (int64_t)me.i + 1] = h[1];
  out[3 * (int64_t)me.i + 2] = h[2];
}

__global__ void __launch_bounds__(kBlock) fields_f64(const __grid_constant__ Params P, const double* __restrict__ s0,
                                                    double* __restrict__ out, int replica) {
  const ReplicaDev* Rp;
  const Me me = whoami(P, Rp);
  if (!me.active || me.r != replica) return;
  const ReplicaDev& R = *Rp;
  const Site st = locate(R, P.nb, me.i);
  const Planes<const double> S = planes(s0, P.npad);
  const double s[3] = {S.x[me.gi], S.y[me.gi], S.z[me.gi]};
  double h[3];
  field_f64(P, R, st, me.gi, S, s, h, P.hdip64, P.pulse_now64);
  out[3 * (int64_t)me.i] = h[0];
  out[3 * (int64_t)me.i + 1] = h[1];
  out[3 * (int64_t)me.i + 2] = h[2];
}

// the field (meV) of term `term` alone, as the reference's
// Hamiltonian::calculate_fields leaves it in field_ (src/jams/core/
// hamiltonian.h:15-78): FP64 in the reference's association order, FP32C
// from the FP32 state with the FP32 term arithmetic; AoS N x 3 doubles
__global__ void __launch_bounds__(kBlock) term_fields_f64(const __grid_constant__ Params P,
                                                         const double* __restrict__ s0, double* __restrict__ out,
                                                         int replica, int term) {
  const ReplicaDev* Rp;
  const Me me = whoami(P, Rp);
  if (!me.active || me.r != replica) return;
  const ReplicaDev& R = *Rp;
  const Site st = locate(R, P.nb, me.i);
  const Planes<const double> S = planes(s0, P.npad);
  const double s[3] = {S.x[me.gi], S.y[me.gi], S.z[me.gi]};
  double f[3];
  term_field_f64(P, P.term[term], R, st, me.gi, S, s, f, P.hdip64, P.pulse_now64);
  out[3 * (int64_t)me.i] = f[0];
  out[3 * (int64_t)me.i + 1] = f[1];
  out[3 * (int64_t)me.i + 2] = f[2];
}

__global__ void __launch_bounds__(kBlock) term_fields_f32(const __grid_constant__ Params P,
                                                         const float* __restrict__ s0, double* __restrict__ out,
                                                         int replica, int term) {
  const ReplicaDev* Rp;
  const Me me = whoami(P, Rp);
  if (!me.active || me.r != replica) return;
  const ReplicaDev& R = *Rp;
  const Site st = locate(R, P.nb, me.i);
  const Planes<const float> S = planes(s0, P.npad);
  const float s[3] = {S.x[me.gi], S.y[me.gi], S.z[me.gi]};
  float h[3];
  field_f32(P, R, st, me.gi, S, s, h, P.hdip32, P.pulse_now32, term);
  out[3 * (int64_t)me.i] = h[0];
  out[3 * (int64_t)me.i + 1] = h[1];
  out[3 * (int64_t)me.i + 2] = h[2];
}

}  // namespace jams_llg

namespace jams_llg {

// host-side launchers for the templated kernels (their stubs are local to
// this translation unit)
void launch_rk4_f32(int stage, unsigned grid, cudaStream_t st, const Params& P, const float* s0, const float* sin,
                    float* acc, float* sout, uint32_t k) {
  switch (stage) {
    case 1: rk4_stage_f32<1><<<grid, kBlock, 0, st>>>(P, s0, sin, acc, sout, k); break;
    case 2: rk4_stage_f32<2><<<grid, kBlock, 0, st>>>(P, s0, sin, acc, sout, k); break;
    case 3: rk4_stage_f32<3><<<grid, kBlock, 0, st>>>(P, s0, sin, acc, sout, k); break;
    default: rk4_stage_f32<4><<<grid, kBlock, 0, st>>>(P, s0, sin, acc, sout, k); break;
  }
}

void launch_rk4_f64(int stage, unsigned grid, cudaStream_t st, const Params& P, const double* s0,
                    const double* sin, double* acc, double* sout, uint32_t k) {
  switch (stage) {
    case 1: rk4_stage_f64<1><<<grid, kBlock, 0, st>>>(P, s0, sin, acc, sout, k); break;
    case 2: rk4_stage_f64<2><<<grid, kBlock, 0, st>>>(P, s0, sin, acc, sout, k); break;
    case 3: rk4_stage_f64<3><<<grid, kBlock, 0, st>>>(P, s0, sin, acc, sout, k); break;
    default: rk4_stage_f64<4><<<grid, kBlock, 0, st>>>(P, s0, sin, acc, sout, k); break;
  }
}

void launch_unpack(bool fp64, cudaStream_t st, const double* aos, void* soa, int64_t offset, int64_t n,
                   int64_t npad) {
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (fp64)
    unpack_state<double><<<grid, 256, 0, st>>>(aos, (double*)soa, offset, n, npad);
  else
    unpack_state<float><<<grid, 256, 0, st>>>(aos, (float*)soa, offset, n, npad);
}

void launch_pack(bool fp64, cudaStream_t st, const void* soa, double* aos, int64_t offset, int64_t n,
                 int64_t npad) {
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (fp64)
    pack_state<double><<<grid, 256, 0, st>>>((const double*)soa, aos, offset, n, npad);
  else
    pack_state<float><<<grid, 256, 0, st>>>((const float*)soa, aos, offset, n, npad);
}

}  // namespace jams_llg
