// Tiled FP32 stage kernels for lattices that match a compile-time stencil
// family (llg_families.h).
//
// 2.5-D streaming: a CTA owns a TY x TZ patch of cells (all basis sites) and
// walks TX planes along the slowest axis X.  The spins of planes x-1, x, x+1
// sit in a four-plane ring of float4 in shared memory (halo rows/columns
// included, periodic wrap or open-boundary zeros applied once at load time);
// the plane x+2 is fetched into registers while plane x is computed and
// stored into the free ring slot before the CTA barrier.  Every neighbour is
// then one 16-byte shared-memory load at a compile-time offset plus three
// adds, and global memory sees each spin once per stage (plus the halo).
//
// Warps are laid out along Z (32 consecutive cells) with the basis site
// uniform per warp, so the per-basis stencil never diverges.
#include <cstdint>
#include <utility>

#include "llg_families.h"
#include "llg_kernels.h"
#include "llg_noise.cuh"

namespace jams_llg {

namespace {

// every FP32 operation below is an explicit intrinsic: the result does not
// depend on how the compiler would contract a given kernel, so all tiling
// choices (stored or recomputed rhs, planes per CTA) agree bit for bit
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ff(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }

__device__ __forceinline__ void two_sum_t(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void acc_add_t(float& hi, float& lo, float c) {
  float s, e;
  two_sum_t(hi, c, s, e);
  hi = s;
  lo = __fadd_rn(lo, e);
}

__device__ __forceinline__ void acc_mad_t(float& hi, float& lo, float jhi, float jlo, float a) {
  const float p = __fmul_rn(jhi, a);
  const float pe = __fmaf_rn(jhi, a, -p);
  float s, e;
  two_sum_t(hi, p, s, e);
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(e, __fmaf_rn(jlo, a, pe)));
}

// thermal field for the FP32 form: Philox4x32-10 words, Box-Muller with the
// special-function unit (log2, sin, cos, rsqrt)
__device__ __forceinline__ void noise_fast(uint64_t seed, uint32_t replica, uint64_t step, uint32_t spin, float amp,
                                           float w[3]) {
  uint32_t c[4] = {spin, replica, (uint32_t)step, (uint32_t)(step >> 32)};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const float u1 = (float)((c[0] >> 8) + 1u) * 0x1.0p-24f;
  const float u2 = (float)((c[2] >> 8) + 1u) * 0x1.0p-24f;
  const float x1 = fmaxf(-1.3862943611198906f * __log2f(u1), 1e-30f);  // -2 ln u1
  const float x2 = fmaxf(-1.3862943611198906f * __log2f(u2), 1e-30f);
  const float r1 = x1 * rsqrtf(x1), r2 = x2 * rsqrtf(x2);
  float s1, c1, s2, c2;
  __sincosf(6.283185307179586f * (float)(c[1] >> 8) * 0x1.0p-24f, &s1, &c1);
  __sincosf(6.283185307179586f * (float)(c[3] >> 8) * 0x1.0p-24f, &s2, &c2);
  w[0] = __fmul_rn(__fmul_rn(amp, r1), c1);
  w[1] = __fmul_rn(__fmul_rn(amp, r1), s1);
  w[2] = __fmul_rn(__fmul_rn(amp, r2), c2);
}


// anisotropy / applied-field terms (everything but the tiled exchange term)
__device__ __forceinline__ void local_terms(const Params& P, const ReplicaDev& R, int b, int skip,
                                            const float s[3], float hi[3], float lo[3]) {
  for (int t = 0; t < P.nterms; ++t) {
    if (t == skip) continue;
    const TermDev& T = P.term[t];
    if (T.kind == kUniaxial) {
      const float* a = T.axisf[b];
      const float d = ff(a[2], s[2], ff(a[1], s[1], fm(a[0], s[0])));
      float pw = d;
      if (T.order >= 4) pw = fm(fm(d, d), d);
      if (T.order >= 6) pw = fm(fm(pw, d), d);
      const float pre = fm(fm(T.Kf[b], (float)T.order), pw);
#pragma unroll
      for (int m = 0; m < 3; ++m) acc_add_t(hi[m], lo[m], fm(pre, a[m]));
    } else if (T.kind == kCubic) {
      const float* u = T.axisf[b];
      const float Su = ff(u[2], s[2], ff(u[1], s[1], fm(u[0], s[0])));
      const float Sv = ff(u[5], s[2], ff(u[4], s[1], fm(u[3], s[0])));
      const float Sw = ff(u[8], s[2], ff(u[7], s[1], fm(u[6], s[0])));
      const float pre = fm(2.0f, T.Kf[b]);
      const float Su2 = fm(Su, Su), Sv2 = fm(Sv, Sv), Sw2 = fm(Sw, Sw);
      float cu, cv, cw;
      if (T.order == 1) {
        cu = fm(Su, fa(Sv2, Sw2));
        cv = fm(Sv, fa(Sw2, Su2));
        cw = fm(Sw, fa(Su2, Sv2));
      } else {
        cu = fm(fm(Su, Sv2), Sw2);
        cv = fm(fm(Sv, Sw2), Su2);
        cw = fm(fm(Sw, Su2), Sv2);
      }
#pragma unroll
      for (int m = 0; m < 3; ++m) acc_add_t(hi[m], lo[m], fm(pre, ff(u[6 + m], cw, ff(u[3 + m], cv, fm(u[m], cu)))));
    } else if (T.kind == kAppliedField) {
#pragma unroll
      for (int m = 0; m < 3; ++m) acc_add_t(hi[m], lo[m], fm(P.mus32[b], R.Bf[m]));
    }
  }
}

__device__ __forceinline__ void llg_rhs_t(const Params& P, int b, const float s[3], const float h[3], const float w[3],
                                          float rhs[3]) {
  const float im = P.inv_mus32[b];
  const float hh[3] = {ff(h[0], im, w[0]), ff(h[1], im, w[1]), ff(h[2], im, w[2])};
  const float c1[3] = {ff(s[1], hh[2], -fm(s[2], hh[1])), ff(s[2], hh[0], -fm(s[0], hh[2])),
                       ff(s[0], hh[1], -fm(s[1], hh[0]))};
  const float c2[3] = {ff(s[1], c1[2], -fm(s[2], c1[1])), ff(s[2], c1[0], -fm(s[0], c1[2])),
                       ff(s[0], c1[1], -fm(s[1], c1[0]))};
  const float mg = -P.gyro32[b], a = P.alpha32[b];
#pragma unroll
  for (int m = 0; m < 3; ++m) rhs[m] = fm(mg, ff(a, c2[m], c1[m]));
}

__device__ __forceinline__ void normalise_t(float v[3]) {
  const float r = rsqrtf(ff(v[2], v[2], ff(v[1], v[1], fm(v[0], v[0]))));
  v[0] = fm(v[0], r);
  v[1] = fm(v[1], r);
  v[2] = fm(v[2], r);
}

template <class F, int TZ, int TY>
struct Geo {
  static constexpr int NB = F::NB;
  static constexpr int PY = TY + 2 * F::RY;
  static constexpr int PZ = TZ + 2 * F::RZ;
  static constexpr int PLANE = NB * PY * PZ;   // float4 per ring slot
  static constexpr int NT = TZ * TY * NB;
  static constexpr int PER_THREAD = (PLANE + NT - 1) / NT;
};

template <class F>
__host__ __device__ constexpr int shell_of(int b, int k) {
  int g = 0;
  while (g + 1 < F::NSHELL && k >= F::shell_end(b, g)) ++g;
  return g;
}

// one neighbour slot: every offset is a compile-time constant
template <class F, int TZ, int TY, int B, int K>
__device__ __forceinline__ void gather_slot(const float4* bm, const float4* b0, const float4* bp,
                                            float (&a)[F::NSHELL][3], float (&r)[3], const TiledParams& TP) {
  using G = Geo<F, TZ, TY>;
  constexpr Slot sl = F::slot(B, K);
  constexpr int off = (sl.bj * G::PY + sl.dy) * G::PZ + sl.dz;
  constexpr int g = shell_of<F>(B, K);
  const float4* p = sl.dx < 0 ? bm : (sl.dx == 0 ? b0 : bp);
  const float4 v = p[off];
  a[g][0] = fa(a[g][0], v.x);
  a[g][1] = fa(a[g][1], v.y);
  a[g][2] = fa(a[g][2], v.z);
  if constexpr (F::REST != 0) {
    const float* J = TP.rest[B][K];
    r[0] = ff(J[0], v.x, ff(J[1], v.y, ff(J[2], v.z, r[0])));
    r[1] = ff(J[3], v.x, ff(J[4], v.y, ff(J[5], v.z, r[1])));
    r[2] = ff(J[6], v.x, ff(J[7], v.y, ff(J[8], v.z, r[2])));
  }
}

template <class F, int TZ, int TY, int B, int... K>
__device__ __forceinline__ void gather_all(std::integer_sequence<int, K...>, const float4* bm, const float4* b0,
                                           const float4* bp, float (&a)[F::NSHELL][3], float (&r)[3],
                                           const TiledParams& TP) {
  (gather_slot<F, TZ, TY, B, K>(bm, b0, bp, a, r, TP), ...);
}

// exchange field of basis site B at the thread's cell from one ring: plain
// FP32 sum of the neighbour spins of each shell, then h += J_shell * sum with
// TwoProd/TwoSum compensation; 3x3 remainders (REST families) per slot
template <class F, int TZ, int TY, int B>
__device__ __forceinline__ void exchange_tiled(const TiledParams& TP, const float4* ring, int xs, int own,
                                               float hi[3], float lo[3]) {
  using G = Geo<F, TZ, TY>;
  const float4* bm = ring + ((xs + 3) & 3) * G::PLANE + own;
  const float4* b0 = ring + (xs & 3) * G::PLANE + own;
  const float4* bp = ring + ((xs + 1) & 3) * G::PLANE + own;
  float a[F::NSHELL][3];
  float r[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int g = 0; g < F::NSHELL; ++g) a[g][0] = a[g][1] = a[g][2] = 0.f;
  gather_all<F, TZ, TY, B>(std::make_integer_sequence<int, F::Z>{}, bm, b0, bp, a, r, TP);
#pragma unroll
  for (int g = 0; g < F::NSHELL; ++g) {
    acc_mad_t(hi[0], lo[0], TP.shell_hi[B][g], TP.shell_lo[B][g], a[g][0]);
    acc_mad_t(hi[1], lo[1], TP.shell_hi[B][g], TP.shell_lo[B][g], a[g][1]);
    acc_mad_t(hi[2], lo[2], TP.shell_hi[B][g], TP.shell_lo[B][g], a[g][2]);
  }
  if constexpr (F::REST != 0) {
    acc_add_t(hi[0], lo[0], r[0]);
    acc_add_t(hi[1], lo[1], r[1]);
    acc_add_t(hi[2], lo[2], r[2]);
  }
}

template <class F, int TZ, int TY>
__device__ __forceinline__ void exchange_dispatch(int b, const TiledParams& TP, const float4* ring, int xs, int own,
                                                  float hi[3], float lo[3]) {
  if (F::NB == 1 || b == 0) {
    exchange_tiled<F, TZ, TY, 0>(TP, ring, xs, own, hi, lo);
  } else if (F::NB > 1) {
    exchange_tiled<F, TZ, TY, (F::NB > 1 ? 1 : 0)>(TP, ring, xs, own, hi, lo);
  }
}

// total field (meV) of the thread's spin from ring `ring`
template <class F, int TZ, int TY>
__device__ __forceinline__ void field_tiled(const Params& P, const TiledParams& TP, const ReplicaDev& R, int b,
                                           const float4* ring, int xs, int own, float h[3], float s[3]) {
  using G = Geo<F, TZ, TY>;
  const float4 c = ring[(xs & 3) * G::PLANE + own + b * G::PY * G::PZ];
  s[0] = c.x;
  s[1] = c.y;
  s[2] = c.z;
  float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
  exchange_dispatch<F, TZ, TY>(b, TP, ring, xs, own, hi, lo);
  local_terms(P, R, b, TP.exch_term, s, hi, lo);
#pragma unroll
  for (int m = 0; m < 3; ++m) h[m] = hi[m] + lo[m];
}

// one ring slot worth of spins for plane x: registers, then shared memory
template <class F, int TZ, int TY>
struct PlaneRegs {
  float v[Geo<F, TZ, TY>::PER_THREAD][3];
};

// the replica's tile view, held in registers for the whole CTA
struct View {
  int L[3];
  int st[3];      // spin-index strides (Z stride = basis count)
  bool per[3];
  int64_t offset;
};

__device__ __forceinline__ View load_view(const ReplicaDev& R) {
  View v;
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    v.L[l] = R.vL[l];
    v.st[l] = (int)R.vs[l];
    v.per[l] = R.vper[l] != 0;
  }
  v.offset = R.offset;
  return v;
}

// periodic wrap of a coordinate within one period of the lattice, without
// branches; `valid` drops to false outside an open boundary or the lattice
__device__ __forceinline__ int wrap_sel(int c, int L, bool per, bool& valid) {
  const bool lo = c < 0, hi = c >= L;
  valid = valid && (per || !(lo || hi));
  const int w = c + (lo ? L : 0) - (hi ? L : 0);
  valid = valid && w >= 0 && w < L;
  return w;
}

template <class F, int TZ, int TY>
__device__ __forceinline__ void fetch_plane(const View& V, const float* __restrict__ s, int64_t npad, int x,
                                            int y0, int z0, int tid, PlaneRegs<F, TZ, TY>& pr) {
  using G = Geo<F, TZ, TY>;
  bool xvalid = true;
  const int gx = wrap_sel(x, V.L[0], V.per[0], xvalid);
  const float* sx = s + V.offset;
#pragma unroll
  for (int q = 0; q < G::PER_THREAD; ++q) {
    const int idx = tid + q * G::NT;
    const int bb = idx % G::NB;
    const int t = idx / G::NB;
    const int zz = t % G::PZ;
    const int yy = t / G::PZ;
    bool valid = xvalid && idx < G::PLANE;
    const int gy = wrap_sel(y0 - F::RY + yy, V.L[1], V.per[1], valid);
    const int gz = wrap_sel(z0 - F::RZ + zz, V.L[2], V.per[2], valid);
    const int i = gx * V.st[0] + gy * V.st[1] + gz * V.st[2] + bb;
    pr.v[q][0] = valid ? __ldg(sx + i) : 0.f;
    pr.v[q][1] = valid ? __ldg(sx + npad + i) : 0.f;
    pr.v[q][2] = valid ? __ldg(sx + 2 * npad + i) : 0.f;
  }
}

template <class F, int TZ, int TY>
__device__ __forceinline__ void store_plane(float4* ring, int x, int tid, const PlaneRegs<F, TZ, TY>& pr) {
  using G = Geo<F, TZ, TY>;
  float4* slot = ring + (x & 3) * G::PLANE;
#pragma unroll
  for (int q = 0; q < G::PER_THREAD; ++q) {
    const int idx = tid + q * G::NT;
    if (idx < G::PLANE) {
      const int bb = idx % G::NB;
      const int t = idx / G::NB;
      const int zz = t % G::PZ;
      const int yy = t / G::PZ;
      slot[(bb * G::PY + yy) * G::PZ + zz] = make_float4(pr.v[q][0], pr.v[q][1], pr.v[q][2], 0.f);
    }
  }
}

}  // namespace

// STAGE: 0 Heun predictor (writes sp; with aux != null also rhs0 into aux)
//        1 Heun corrector recomputing rhs(s0) (rings of s0 and sp)
//        2 Heun corrector from stored rhs0 (ring of sp; own s0 and aux)
//        3..6 RK4 stages 1..4 (ring of sin; own s0, aux = k accumulator)
template <class F, int TZ, int TY, int STAGE>
__global__ void __launch_bounds__(Geo<F, TZ, TY>::NT) tiled_stage(const __grid_constant__ Params P,
                                                                  const __grid_constant__ TiledParams TP,
                                                                  const float* s0, const float* sin, float* out,
                                                                  float* aux, uint32_t kstep) {
  using G = Geo<F, TZ, TY>;
  constexpr int NR = STAGE == 1 ? 2 : 1;
  extern __shared__ float4 smem[];
  float4* ring0 = smem;                    // ring of the gathered state
  float4* ring1 = smem + 4 * G::PLANE;     // second ring (s0) for STAGE 1
  const int4 tile = TP.tiles[blockIdx.x];
  const ReplicaDev& R = P.rep[tile.x];
  const View V = load_view(R);
  const int thermal = R.thermal;
  const int x0 = tile.y, y0 = tile.z, z0 = tile.w;
  const int tid = threadIdx.x + TZ * threadIdx.y;
  const int tz = threadIdx.x;
  const int ty = threadIdx.y % TY;
  const int b = threadIdx.y / TY;
  const float amp = R.amp32[b];
  const int y = y0 + ty, z = z0 + tz;
  const bool active_yz = y < V.L[1] && z < V.L[2];
  const int own = (ty + F::RY) * G::PZ + (tz + F::RZ);
  const uint64_t step = *P.step_base + kstep;
  const float* gather_src = STAGE == 0 ? s0 : sin;
  const int xe = min(x0 + TP.TX, V.L[0]);

  {
    PlaneRegs<F, TZ, TY> pr;
#pragma unroll
    for (int d = -1; d <= 1; ++d) {
      fetch_plane<F, TZ, TY>(V, gather_src, P.npad, x0 + d, y0, z0, tid, pr);
      store_plane<F, TZ, TY>(ring0, x0 + d, tid, pr);
      if (NR == 2) {
        fetch_plane<F, TZ, TY>(V, s0, P.npad, x0 + d, y0, z0, tid, pr);
        store_plane<F, TZ, TY>(ring1, x0 + d, tid, pr);
      }
    }
  }
  __syncthreads();

  for (int x = x0; x < xe; ++x) {
    const bool more = x + 1 < xe;
    PlaneRegs<F, TZ, TY> pf0, pf1;
    if (more) {
      fetch_plane<F, TZ, TY>(V, gather_src, P.npad, x + 2, y0, z0, tid, pf0);
      if (NR == 2) fetch_plane<F, TZ, TY>(V, s0, P.npad, x + 2, y0, z0, tid, pf1);
    }
    if (active_yz) {
      const int i = x * V.st[0] + y * V.st[1] + z * V.st[2] + b;  // spin index in the replica
      const int64_t gi = V.offset + i;
      float w[3] = {0.f, 0.f, 0.f};
      if (thermal) noise_fast(P.seed, (uint32_t)tile.x, step, (uint32_t)i, amp, w);
      float h[3], s[3], k[3];
      field_tiled<F, TZ, TY>(P, TP, R, b, ring0, x, own, h, s);
      llg_rhs_t(P, b, s, h, w, k);
      if (STAGE == 0) {
        float v[3] = {__fmaf_rn(P.dt32, k[0], s[0]), __fmaf_rn(P.dt32, k[1], s[1]), __fmaf_rn(P.dt32, k[2], s[2])};
        normalise_t(v);
        out[gi] = v[0];
        out[P.npad + gi] = v[1];
        out[2 * P.npad + gi] = v[2];
        if (aux) {
          aux[gi] = k[0];
          aux[P.npad + gi] = k[1];
          aux[2 * P.npad + gi] = k[2];
        }
      } else if (STAGE == 1 || STAGE == 2) {
        float a[3], r0[3];
        if (STAGE == 1) {
          float h0[3];
          field_tiled<F, TZ, TY>(P, TP, R, b, ring1, x, own, h0, a);
          llg_rhs_t(P, b, a, h0, w, r0);
        } else {
          a[0] = s0[gi];
          a[1] = s0[P.npad + gi];
          a[2] = s0[2 * P.npad + gi];
          r0[0] = aux[gi];
          r0[1] = aux[P.npad + gi];
          r0[2] = aux[2 * P.npad + gi];
        }
        const float hdt = fm(0.5f, P.dt32);
        float v[3] = {ff(hdt, fa(r0[0], k[0]), a[0]), ff(hdt, fa(r0[1], k[1]), a[1]),
                      ff(hdt, fa(r0[2], k[2]), a[2])};
        normalise_t(v);
        if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) atomicOr(P.status, 1u);
        out[gi] = v[0];
        out[P.npad + gi] = v[1];
        out[2 * P.npad + gi] = v[2];
      } else {
        const float a[3] = {s0[gi], s0[P.npad + gi], s0[2 * P.npad + gi]};
        float v[3];
        if (STAGE == 6) {
          const float c = fm(P.dt32, 1.0f / 6.0f);
#pragma unroll
          for (int m = 0; m < 3; ++m) v[m] = ff(c, fa(aux[m * P.npad + gi], k[m]), a[m]);
          normalise_t(v);
          if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) atomicOr(P.status, 1u);
        } else {
          const float c = STAGE == 5 ? P.dt32 : fm(0.5f, P.dt32);
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            const float acc = STAGE == 3 ? k[m] : __fmaf_rn(2.0f, k[m], aux[m * P.npad + gi]);
            aux[m * P.npad + gi] = acc;
            v[m] = __fmaf_rn(c, k[m], a[m]);
          }
          if (P.rk4_normalise_stages) normalise_t(v);
        }
        out[gi] = v[0];
        out[P.npad + gi] = v[1];
        out[2 * P.npad + gi] = v[2];
      }
    }
    if (more) {
      store_plane<F, TZ, TY>(ring0, x + 2, tid, pf0);
      if (NR == 2) store_plane<F, TZ, TY>(ring1, x + 2, tid, pf1);
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ launchers --

namespace {

template <class F, int TZ, int TY>
size_t smem_bytes(int stage) {
  return (size_t)(stage == 1 ? 2 : 1) * 4 * Geo<F, TZ, TY>::PLANE * sizeof(float4);
}

template <class F, int TZ, int TY, int STAGE>
cudaError_t launch_one(unsigned grid, cudaStream_t st, const Params& P, const TiledParams& TP, const float* s0,
                       const float* sin, float* out, float* aux, uint32_t k) {
  const size_t sm = smem_bytes<F, TZ, TY>(STAGE);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(tiled_stage<F, TZ, TY, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sm);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const dim3 block(TZ, TY * F::NB);
  tiled_stage<F, TZ, TY, STAGE><<<grid, block, sm, st>>>(P, TP, s0, sin, out, aux, k);
  return cudaSuccess;
}

template <class F, int TZ, int TY>
cudaError_t launch_family(int stage, unsigned grid, cudaStream_t st, const Params& P, const TiledParams& TP,
                          const float* s0, const float* sin, float* out, float* aux, uint32_t k) {
  switch (stage) {
    case 0: return launch_one<F, TZ, TY, 0>(grid, st, P, TP, s0, sin, out, aux, k);
    case 1: return launch_one<F, TZ, TY, 1>(grid, st, P, TP, s0, sin, out, aux, k);
    case 2: return launch_one<F, TZ, TY, 2>(grid, st, P, TP, s0, sin, out, aux, k);
    case 3: return launch_one<F, TZ, TY, 3>(grid, st, P, TP, s0, sin, out, aux, k);
    case 4: return launch_one<F, TZ, TY, 4>(grid, st, P, TP, s0, sin, out, aux, k);
    case 5: return launch_one<F, TZ, TY, 5>(grid, st, P, TP, s0, sin, out, aux, k);
    default: return launch_one<F, TZ, TY, 6>(grid, st, P, TP, s0, sin, out, aux, k);
  }
}

}  // namespace

void tiled_geometry(int family, int* tz, int* ty) {
  switch (family) {
    case kFamSC: *tz = 32; *ty = 8; break;
    case kFamBCC:
    case kFamBCC3: *tz = 32; *ty = 4; break;
    case kFamTRI: *tz = 256; *ty = 1; break;
    default: *tz = 0; *ty = 0; break;
  }
}

cudaError_t launch_tiled(int family, int stage, unsigned grid, cudaStream_t st, const Params& P, const TiledParams& TP,
                         const float* s0, const float* sin, float* out, float* aux, uint32_t k) {
  switch (family) {
    case kFamSC: return launch_family<FamSC, 32, 8>(stage, grid, st, P, TP, s0, sin, out, aux, k);
    case kFamBCC: return launch_family<FamBCC, 32, 4>(stage, grid, st, P, TP, s0, sin, out, aux, k);
    case kFamBCC3: return launch_family<FamBCC3, 32, 4>(stage, grid, st, P, TP, s0, sin, out, aux, k);
    case kFamTRI: return launch_family<FamTRI, 256, 1>(stage, grid, st, P, TP, s0, sin, out, aux, k);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace jams_llg
