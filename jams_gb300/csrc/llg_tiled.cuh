// Tiled FP32 stage kernels for lattices that match a compile-time stencil
// family (llg_families.h).  Implementation header, compiled in parallel by
// llg_tiled.cu (one row per thread, no dipole term), llg_tiled_dipole.cu
// (DIP: the dipole field planes are read and added) and llg_tiled_pair.cu
// (two rows per thread).
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
#pragma once
#include <cuda.h>

#include <cstdint>
#include <type_traits>
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

// packed pairs of FP32 (Blackwell f32x2 instructions, round to nearest):
// the x and y components of a spin or field travel as one 64-bit register
// (the 64-bit pairs are formed and split inside the PTX, so no C++ type
// punning is involved)
#define JAMS_F32X2_BINARY(NAME, OP)                                                              \
  __device__ __forceinline__ float2 NAME(float2 a, float2 b) {                                    \
    float2 d;                                                                                     \
    asm("{.reg .b64 ra, rb, rd;\n\t"                                                              \
        "mov.b64 ra, {%2, %3};\n\t"                                                               \
        "mov.b64 rb, {%4, %5};\n\t" OP " rd, ra, rb;\n\t"                                       \
        "mov.b64 {%0, %1}, rd;}"                                                                  \
        : "=f"(d.x), "=f"(d.y)                                                                    \
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                                \
    return d;                                                                                     \
  }
JAMS_F32X2_BINARY(add2, "add.rn.f32x2")
JAMS_F32X2_BINARY(sub2, "sub.rn.f32x2")
JAMS_F32X2_BINARY(mul2, "mul.rn.f32x2")
#undef JAMS_F32X2_BINARY

__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\t"
      "mov.b64 rb, {%4, %5};\n\t"
      "mov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\t"
      "mov.b64 {%0, %1}, rd;}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}

// (hi, lo) += (jhi + jlo) a for a packed pair, with TwoProd (p = jhi a,
// pe = jhi a - p exactly) and TwoSum (hi + p = s + e exactly); jn = -jhi
// lets the negated product feed both without extra sign flips
__device__ __forceinline__ void acc_mad2(float2& hi, float2& lo, float jhi, float jn, float jlo, float2 a) {
  const float2 J = make_float2(jhi, jhi), JN = make_float2(jn, jn), JL = make_float2(jlo, jlo);
  const float2 pn = mul2(JN, a);         // -p
  const float2 pe = fma2(J, a, pn);      // jhi a - p
  const float2 s = sub2(hi, pn);         // hi + p
  const float2 bb = sub2(s, hi);
  const float2 e = sub2(sub2(hi, sub2(s, bb)), add2(pn, bb));
  hi = s;
  lo = add2(lo, add2(e, fma2(JL, a, pe)));
}

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

// thermal field for the FP32 form, Box-Muller with the special-function
// unit (log2, sin, cos, rsqrt): two spins (planes x and x + 1 of one column,
// x even) from one Philox4x32-10 call keyed by the even spin's index; six
// 21-bit uniforms (the four words' top 21 bits, and their low bits
// recombined) make three Box-Muller pairs.  The largest normal is
// sqrt(-2 ln 2^-21) = 5.4.
__device__ __forceinline__ float bm_radius(uint32_t k) {
  const float u = (float)(k + 1u) * 0x1.0p-21f;  // (0, 1]
  const float x = fmaxf(-1.3862943611198906f * __log2f(u), 1e-30f);  // -2 ln u
  return x * rsqrtf(x);
}

__device__ __forceinline__ void noise_pair(const uint32_t* keys, uint32_t replica, uint64_t step, uint32_t spin,
                                           float amp, float wa[3], float wb[3]) {
  uint32_t c[4] = {spin, replica, (uint32_t)step, (uint32_t)(step >> 32)};
  philox4x32_10_keyed(c, keys);
  const uint32_t k4 = ((c[0] & 0x7FFu) << 10) | (c[1] & 0x3FFu);
  const uint32_t k5 = ((c[2] & 0x7FFu) << 10) | (c[3] & 0x3FFu);
  const float r0 = fm(amp, bm_radius(c[0] >> 11)), r1 = fm(amp, bm_radius(c[2] >> 11)), r2 = fm(amp, bm_radius(k4));
  float s0, c0, s1, c1, s2, c2;
  __sincosf(6.283185307179586f * (float)(c[1] >> 11) * 0x1.0p-21f, &s0, &c0);
  __sincosf(6.283185307179586f * (float)(c[3] >> 11) * 0x1.0p-21f, &s1, &c1);
  __sincosf(6.283185307179586f * (float)k5 * 0x1.0p-21f, &s2, &c2);
  wa[0] = fm(r0, c0);
  wa[1] = fm(r0, s0);
  wa[2] = fm(r1, c1);
  wb[0] = fm(r1, s1);
  wb[1] = fm(r2, c2);
  wb[2] = fm(r2, s2);
}

// Anisotropy and applied-field terms of one basis site, gathered once per
// CTA into registers (at most one uniaxial, one cubic and one applied-field
// term; the host sends other term lists to the gather kernels).  They are
// summed in plain FP32 and added to the low word of the compensated
// exchange sum.
struct LocalField {
  float uk;       // K * p of the uniaxial term (0: none)
  int upow;
  float ua[3];
  float ck;       // 2 K of the cubic term (0: none)
  int corder;
  float cu[9];
  float hb[3];    // mu_s B of the applied-field and zeeman terms
  float inv_mus, mg, alpha;
};

// mu_s B of the applied-field term (times the pulse factors) plus the zeeman
// term's mu_s B_dc + mu_s B_ac cos(w t), at the time factors pf (null: none)
__device__ __forceinline__ void field_terms_hb(const Params& P, const ReplicaDev& R, int b, const float* pf,
                                               float hb[3]) {
  hb[0] = hb[1] = hb[2] = 0.f;
#pragma unroll 1
  for (int t = 0; t < P.nterms; ++t) {
    const TermDev& T = P.term[t];
    if (T.kind == kAppliedField) {
      for (int m = 0; m < 3; ++m) hb[m] = fa(hb[m], fm(P.mus32[b], pf ? fm(fm(R.Bf[m], pf[0]), pf[1]) : R.Bf[m]));
    } else if (T.kind == kZeeman) {
      for (int m = 0; m < 3; ++m)
        hb[m] = fa(hb[m], (T.order && pf) ? ff(T.axisf[b][3 + m], pf[2 + b], T.axisf[b][m]) : T.axisf[b][m]);
    }
  }
}

__device__ __forceinline__ LocalField local_field(const Params& P, const ReplicaDev& R, int b, int skip) {
  LocalField L;
  L.uk = 0.f;
  L.upow = 2;
  L.ck = 0.f;
  L.corder = 1;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    L.ua[m] = 0.f;
    L.hb[m] = 0.f;
  }
#pragma unroll
  for (int m = 0; m < 9; ++m) L.cu[m] = 0.f;
  for (int t = 0; t < P.nterms; ++t) {
    if (t == skip) continue;
    const TermDev& T = P.term[t];
    if (T.kind == kUniaxial) {
      L.uk = fm(T.Kf[b], (float)T.order);
      L.upow = T.order;
      for (int m = 0; m < 3; ++m) L.ua[m] = T.axisf[b][m];
    } else if (T.kind == kCubic) {
      L.ck = fm(2.0f, T.Kf[b]);
      L.corder = T.order;
      for (int m = 0; m < 9; ++m) L.cu[m] = T.axisf[b][m];
    }
  }
  // L.hb: field_terms_hb once the stage's time is known
  L.inv_mus = P.inv_mus32[b];
  L.mg = -P.gyro32[b];
  L.alpha = P.alpha32[b];
  return L;
}

__device__ __forceinline__ void local_terms(const LocalField& L, const float s[3], float hi[3], float lo[3]) {
  float l[3] = {L.hb[0], L.hb[1], L.hb[2]};
  if (L.uk != 0.f) {
    const float d = ff(L.ua[2], s[2], ff(L.ua[1], s[1], fm(L.ua[0], s[0])));
    float pw = d;
    if (L.upow >= 4) pw = fm(fm(d, d), d);
    if (L.upow >= 6) pw = fm(fm(pw, d), d);
    const float pre = fm(L.uk, pw);
#pragma unroll
    for (int m = 0; m < 3; ++m) l[m] = ff(pre, L.ua[m], l[m]);
  }
  if (L.ck != 0.f) {
    const float* u = L.cu;
    const float Su = ff(u[2], s[2], ff(u[1], s[1], fm(u[0], s[0])));
    const float Sv = ff(u[5], s[2], ff(u[4], s[1], fm(u[3], s[0])));
    const float Sw = ff(u[8], s[2], ff(u[7], s[1], fm(u[6], s[0])));
    const float Su2 = fm(Su, Su), Sv2 = fm(Sv, Sv), Sw2 = fm(Sw, Sw);
    float cu, cv, cw;
    if (L.corder == 1) {
      cu = fm(Su, fa(Sv2, Sw2));
      cv = fm(Sv, fa(Sw2, Su2));
      cw = fm(Sw, fa(Su2, Sv2));
    } else {
      cu = fm(fm(Su, Sv2), Sw2);
      cv = fm(fm(Sv, Sw2), Su2);
      cw = fm(fm(Sw, Su2), Sv2);
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) l[m] = ff(L.ck, ff(u[6 + m], cw, ff(u[3 + m], cv, fm(u[m], cu))), l[m]);
  }
  // these terms are small next to the exchange field: added to the low
  // word, their rounding stays at their own magnitude
#pragma unroll
  for (int m = 0; m < 3; ++m) lo[m] = fa(lo[m], l[m]);
}

__device__ __forceinline__ void llg_rhs_t(const LocalField& L, const float s[3], const float h[3], const float w[3],
                                          float rhs[3]) {
  const float im = L.inv_mus;
  const float hh[3] = {ff(h[0], im, w[0]), ff(h[1], im, w[1]), ff(h[2], im, w[2])};
  const float c1[3] = {ff(s[1], hh[2], -fm(s[2], hh[1])), ff(s[2], hh[0], -fm(s[0], hh[2])),
                       ff(s[0], hh[1], -fm(s[1], hh[0]))};
  const float c2[3] = {ff(s[1], c1[2], -fm(s[2], c1[1])), ff(s[2], c1[0], -fm(s[0], c1[2])),
                       ff(s[0], c1[1], -fm(s[1], c1[0]))};
  const float mg = L.mg, a = L.alpha;
#pragma unroll
  for (int m = 0; m < 3; ++m) rhs[m] = fm(mg, ff(a, c2[m], c1[m]));
}

__device__ __forceinline__ void normalise_t(float v[3]) {
  const float r = rsqrtf(ff(v[2], v[2], ff(v[1], v[1], fm(v[0], v[0]))));
  v[0] = fm(v[0], r);
  v[1] = fm(v[1], r);
  v[2] = fm(v[2], r);
}

// CTA tile of TZ x TY cells (all basis sites); each thread computes RPT
// consecutive rows of one column (the ring layout does not depend on RPT)
template <class F, int TZ, int TY, int RPT = 1>
struct Geo {
  static constexpr int NB = F::NB;
  static constexpr int PY = TY + 2 * F::RY;
  static constexpr int PZ = TZ + 2 * F::RZ;
  static constexpr int PLANE = NB * PY * PZ;   // float4 per ring slot
  static constexpr int NT = TZ * (TY / RPT) * NB;
  static constexpr int PER_THREAD = (PLANE + NT - 1) / NT;
};

template <class F>
__host__ __device__ constexpr int shell_of(int b, int k) {
  int g = 0;
  while (g + 1 < F::NSHELL && k >= F::shell_end(b, g)) ++g;
  return g;
}

// one neighbour slot: every offset is a compile-time constant.  PK: the
// x and y sums as one packed f32x2 add (the same sums bit for bit as two
// scalar adds; fewer instructions, but in the one-row and fcc kernels the
// packed operands cost registers and spills, so those add scalars)
template <class F, int TZ, int TY, int B, int K, bool PK = false>
__device__ __forceinline__ void gather_slot(const float4* bm, const float4* b0, const float4* bp,
                                            float2 (&axy)[F::NSHELL], float (&az)[F::NSHELL], float (&r)[3],
                                            const TiledParams& TP) {
  using G = Geo<F, TZ, TY>;
  constexpr Slot sl = F::slot(B, K);
  constexpr int off = (sl.bj * G::PY + sl.dy) * G::PZ + sl.dz;
  constexpr int g = shell_of<F>(B, K);
  const float4* p = sl.dx < 0 ? bm : (sl.dx == 0 ? b0 : bp);
  const float4 v = p[off];
  if constexpr (PK) {
    axy[g] = add2(axy[g], make_float2(v.x, v.y));
  } else {
    axy[g].x = fa(axy[g].x, v.x);
    axy[g].y = fa(axy[g].y, v.y);
  }
  az[g] = fa(az[g], v.z);
  if constexpr (F::REST != 0) {
    const float* J = TP.rest[B][K];
    r[0] = ff(J[0], v.x, ff(J[1], v.y, ff(J[2], v.z, r[0])));
    r[1] = ff(J[3], v.x, ff(J[4], v.y, ff(J[5], v.z, r[1])));
    r[2] = ff(J[6], v.x, ff(J[7], v.y, ff(J[8], v.z, r[2])));
  }
}

template <class F, int TZ, int TY, int B, bool PK = false, int... K>
__device__ __forceinline__ void gather_all(std::integer_sequence<int, K...>, const float4* bm, const float4* b0,
                                           const float4* bp, float2 (&axy)[F::NSHELL], float (&az)[F::NSHELL],
                                           float (&r)[3], const TiledParams& TP) {
  (gather_slot<F, TZ, TY, B, K, PK>(bm, b0, bp, axy, az, r, TP), ...);
}

// Separable bcc stencils.  Shell 1 of basis site 0 is the 2x2 block
// (y-1..y, z-1..z) of sublattice 1 in planes x-1 and x; of site 1 the block
// (y..y+1, z..z+1) of sublattice 0 in planes x and x+1.  Shells 2 and 3 (same
// sublattice) are s(x-1) + s(x+1) + E(x) and E(x-1) + E(x+1) + D(x), with E
// the in-plane cross (y +- 1, z +- 1) and D the in-plane diagonals.  Each
// thread walks its column along x, so the block sum Q of the plane behind
// and the cross sums E(x-1), E(x) are carried in registers from the previous
// plane: per spin 4 (bcc) or 14 (3 shells) shared loads instead of 8 or 26.
// The carried values are the same function of the plane data however the
// planes are tiled, so all tilings still agree bit for bit.
struct Carry {
  float q[3];    // shell-1 block sum of the plane behind
  float em[3];   // E(x - 1)
  float e0[3];   // E(x)
};

template <class F, int TZ, int TY, int B>
__device__ __forceinline__ void bcc_block(const float4* p, float q[3]) {
  using G = Geo<F, TZ, TY>;
  constexpr int bj = 1 - B;
  constexpr int d = B == 0 ? -1 : 0;
  const float4 a = p[(bj * G::PY + d) * G::PZ + d];
  const float4 b = p[(bj * G::PY + d) * G::PZ + d + 1];
  const float4 c = p[(bj * G::PY + d + 1) * G::PZ + d];
  const float4 e = p[(bj * G::PY + d + 1) * G::PZ + d + 1];
  q[0] = fa(fa(a.x, b.x), fa(c.x, e.x));
  q[1] = fa(fa(a.y, b.y), fa(c.y, e.y));
  q[2] = fa(fa(a.z, b.z), fa(c.z, e.z));
}

template <class F, int TZ, int TY, int B>
__device__ __forceinline__ void bcc_cross(const float4* p, float e[3]) {
  using G = Geo<F, TZ, TY>;
  const float4 a = p[(B * G::PY + 1) * G::PZ];
  const float4 b = p[(B * G::PY - 1) * G::PZ];
  const float4 c = p[B * G::PY * G::PZ + 1];
  const float4 d = p[B * G::PY * G::PZ - 1];
  e[0] = fa(fa(a.x, b.x), fa(c.x, d.x));
  e[1] = fa(fa(a.y, b.y), fa(c.y, d.y));
  e[2] = fa(fa(a.z, b.z), fa(c.z, d.z));
}

template <class F, int TZ, int TY, int B>
__device__ __forceinline__ void bcc_diag(const float4* p, float e[3]) {
  using G = Geo<F, TZ, TY>;
  const float4 a = p[(B * G::PY + 1) * G::PZ + 1];
  const float4 b = p[(B * G::PY + 1) * G::PZ - 1];
  const float4 c = p[(B * G::PY - 1) * G::PZ + 1];
  const float4 d = p[(B * G::PY - 1) * G::PZ - 1];
  e[0] = fa(fa(a.x, b.x), fa(c.x, d.x));
  e[1] = fa(fa(a.y, b.y), fa(c.y, d.y));
  e[2] = fa(fa(a.z, b.z), fa(c.z, d.z));
}

// the carried sums for the first plane x0 of a tile (ring holds x0-1..x0+1)
template <class F, int TZ, int TY, int B>
__device__ __forceinline__ void carry_init_b(const float4* ring, int xs, int own, Carry& c) {
  using G = Geo<F, TZ, TY>;
  if constexpr (F::SEP != 0) {
    const float4* bm = ring + ((xs + 3) & 3) * G::PLANE + own;
    const float4* b0 = ring + (xs & 3) * G::PLANE + own;
    bcc_block<F, TZ, TY, B>(B == 0 ? bm : b0, c.q);
    if constexpr (F::SEP == 2) {
      bcc_cross<F, TZ, TY, B>(bm, c.em);
      bcc_cross<F, TZ, TY, B>(b0, c.e0);
    }
  }
}

template <class F, int TZ, int TY>
__device__ __forceinline__ void carry_init(int b, const float4* ring, int xs, int own, Carry& c) {
  if constexpr (F::SEP != 0) {
    if (b == 0) carry_init_b<F, TZ, TY, 0>(ring, xs, own, c);
    else carry_init_b<F, TZ, TY, 1>(ring, xs, own, c);
  }
}

template <class F, int B>
__device__ __forceinline__ void shell_combine(const TiledParams& TP, const float2 (&axy)[F::NSHELL],
                                              const float (&az)[F::NSHELL], const float (&r)[3], float hi[3],
                                              float lo[3]);

// exchange field of basis site B at the thread's cell from one ring: plain
// FP32 sum of the neighbour spins of each shell (x and y packed), then
// h += J_shell * sum with TwoProd/TwoSum compensation; 3x3 remainders (REST
// families) per slot
template <class F, int TZ, int TY, int B, bool PK = false>
__device__ __forceinline__ void exchange_tiled(const TiledParams& TP, const float4* ring, int xs, int own,
                                               Carry& cy, float hi[3], float lo[3]) {
  using G = Geo<F, TZ, TY>;
  const float4* bm = ring + ((xs + 3) & 3) * G::PLANE + own;
  const float4* b0 = ring + (xs & 3) * G::PLANE + own;
  const float4* bp = ring + ((xs + 1) & 3) * G::PLANE + own;
  float2 axy[F::NSHELL];
  float az[F::NSHELL];
  float r[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int g = 0; g < F::NSHELL; ++g) {
    axy[g] = make_float2(0.f, 0.f);
    az[g] = 0.f;
  }
  if constexpr (F::SEP != 0) {
    // shell 1: carried block sum of the plane behind + this one's
    float qn[3];
    bcc_block<F, TZ, TY, B>(B == 0 ? b0 : bp, qn);
    axy[0] = make_float2(fa(cy.q[0], qn[0]), fa(cy.q[1], qn[1]));
    az[0] = fa(cy.q[2], qn[2]);
#pragma unroll
    for (int m = 0; m < 3; ++m) cy.q[m] = qn[m];
    if constexpr (F::SEP == 2) {
      float en[3], d0[3];
      bcc_cross<F, TZ, TY, B>(bp, en);
      bcc_diag<F, TZ, TY, B>(b0, d0);
      const float4 sm = bm[B * G::PY * G::PZ];
      const float4 sp = bp[B * G::PY * G::PZ];
      axy[1] = make_float2(fa(fa(sm.x, sp.x), cy.e0[0]), fa(fa(sm.y, sp.y), cy.e0[1]));
      az[1] = fa(fa(sm.z, sp.z), cy.e0[2]);
      axy[2] = make_float2(fa(fa(cy.em[0], en[0]), d0[0]), fa(fa(cy.em[1], en[1]), d0[1]));
      az[2] = fa(fa(cy.em[2], en[2]), d0[2]);
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        cy.em[m] = cy.e0[m];
        cy.e0[m] = en[m];
      }
    }
  } else {
    gather_all<F, TZ, TY, B, PK>(std::make_integer_sequence<int, F::Z>{}, bm, b0, bp, axy, az, r, TP);
  }
  shell_combine<F, B>(TP, axy, az, r, hi, lo);
}

// h = sum over shells of J_shell * (neighbour sum of the shell), compensated:
// the first shell's (hi, lo) is the exact product J a (TwoProd) plus the J
// low word, no TwoSum needed; the other shells are added with TwoSum; the
// 3x3 remainders (REST families) last
template <class F, int B>
__device__ __forceinline__ void shell_combine(const TiledParams& TP, const float2 (&axy)[F::NSHELL],
                                              const float (&az)[F::NSHELL], const float (&r)[3], float hi[3],
                                              float lo[3]) {
  float2 hxy, lxy;
  {
    const float2 J = make_float2(TP.shell_hi[B][0], TP.shell_hi[B][0]);
    const float2 JN = make_float2(-TP.shell_hi[B][0], -TP.shell_hi[B][0]);
    const float2 JL = make_float2(TP.shell_lo[B][0], TP.shell_lo[B][0]);
    const float2 pn = mul2(JN, axy[0]);
    hxy = make_float2(-pn.x, -pn.y);
    lxy = fma2(JL, axy[0], fma2(J, axy[0], pn));
    const float p = fm(TP.shell_hi[B][0], az[0]);
    hi[2] = p;
    lo[2] = ff(TP.shell_lo[B][0], az[0], ff(TP.shell_hi[B][0], az[0], -p));
  }
#pragma unroll
  for (int g = 1; g < F::NSHELL; ++g) {
    acc_mad2(hxy, lxy, TP.shell_hi[B][g], -TP.shell_hi[B][g], TP.shell_lo[B][g], axy[g]);
    acc_mad_t(hi[2], lo[2], TP.shell_hi[B][g], TP.shell_lo[B][g], az[g]);
  }
  hi[0] = hxy.x;
  hi[1] = hxy.y;
  lo[0] = lxy.x;
  lo[1] = lxy.y;
  if constexpr (F::REST != 0) {
    acc_add_t(hi[0], lo[0], r[0]);
    acc_add_t(hi[1], lo[1], r[1]);
    acc_add_t(hi[2], lo[2], r[2]);
  }
}

template <class F, int TZ, int TY, bool PK = false>
__device__ __forceinline__ void exchange_dispatch(int b, const TiledParams& TP, const float4* ring, int xs, int own,
                                                  Carry& cy, float hi[3], float lo[3]) {
  // the basis site is uniform per warp; one compile-time stencil per site
  if (F::NB == 1 || b == 0) {
    exchange_tiled<F, TZ, TY, 0, PK>(TP, ring, xs, own, cy, hi, lo);
  } else if (b == 1) {
    exchange_tiled<F, TZ, TY, (F::NB > 1 ? 1 : 0), PK>(TP, ring, xs, own, cy, hi, lo);
  } else if (b == 2) {
    exchange_tiled<F, TZ, TY, (F::NB > 2 ? 2 : 0), PK>(TP, ring, xs, own, cy, hi, lo);
  } else {
    exchange_tiled<F, TZ, TY, (F::NB > 3 ? 3 : 0), PK>(TP, ring, xs, own, cy, hi, lo);
  }
  static_assert(F::NB <= 4, "at most four basis sites per family");
}

// total field (meV) of the thread's spin from ring `ring`
template <class F, int TZ, int TY, bool PK = false>
__device__ __forceinline__ void field_tiled(const LocalField& L, const TiledParams& TP, int b, const float4* ring,
                                           int xs, int own, Carry& cy, float h[3], float s[3], bool has_dip,
                                           const float dip[3]) {
  using G = Geo<F, TZ, TY>;
  const float4 c = ring[(xs & 3) * G::PLANE + own + b * G::PY * G::PZ];
  s[0] = c.x;
  s[1] = c.y;
  s[2] = c.z;
  float hi[3], lo[3];
  exchange_dispatch<F, TZ, TY, PK>(b, TP, ring, xs, own, cy, hi, lo);
  local_terms(L, s, hi, lo);
  if (has_dip) {   // the dipole field of this spin, precomputed by FFT convolution
#pragma unroll
    for (int m = 0; m < 3; ++m) lo[m] = fa(lo[m], dip[m]);
  }
#pragma unroll
  for (int m = 0; m < 3; ++m) h[m] = hi[m] + lo[m];
}

// one ring slot worth of spins for plane x: registers, then shared memory
template <class F, int TZ, int TY, int RPT>
struct PlaneRegs {
  float v[Geo<F, TZ, TY, RPT>::PER_THREAD][3];
};

// the replica's tile view, held in registers for the whole CTA
struct View {
  int L[3];
  int st[3];      // spin-index strides (Z stride = basis count)
  bool per[3];
  int64_t offset;
};

// a value that is the same in every lane, taken from lane 0: the compiler
// then knows it is warp-uniform and can keep it in a uniform register.
// U = false leaves it in ordinary registers (the two-rows-per-thread kernels
// measured faster that way: their register allocation spilled more with the
// per-CTA view in uniform registers).
template <bool U = true, typename T>
__device__ __forceinline__ T uniform(T v) {
  if constexpr (U) return __shfl_sync(0xffffffffu, v, 0);
  else return v;
}

template <bool U>
__device__ __forceinline__ View load_view(const ReplicaDev& R) {
  View v;
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    v.L[l] = uniform<U>(R.vL[l]);
    v.st[l] = uniform<U>((int)R.vs[l]);
    v.per[l] = uniform<U>(R.vper[l]) != 0;
  }
  v.offset = uniform<U>((long long)R.offset);
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

// the part of a thread's halo loads that does not change from plane to
// plane: which (row, column, basis site) it loads and where it stores it
template <class F, int TZ, int TY, int RPT>
struct FetchPlan {
  int idx[Geo<F, TZ, TY, RPT>::PER_THREAD];   // spin index in the plane (-1: zero / unused)
  int dst[Geo<F, TZ, TY, RPT>::PER_THREAD];   // ring slot offset
};

template <class F, int TZ, int TY, int RPT>
__device__ __forceinline__ void plan_fetch(const View& V, int y0, int z0, int tid, FetchPlan<F, TZ, TY, RPT>& fp) {
  using G = Geo<F, TZ, TY, RPT>;
#pragma unroll
  for (int q = 0; q < G::PER_THREAD; ++q) {
    const int idx = tid + q * G::NT;
    const int bb = idx % G::NB;
    const int t = idx / G::NB;
    const int zz = t % G::PZ;
    const int yy = t / G::PZ;
    bool valid = idx < G::PLANE;
    const int gy = wrap_sel(y0 - F::RY + yy, V.L[1], V.per[1], valid);
    const int gz = wrap_sel(z0 - F::RZ + zz, V.L[2], V.per[2], valid);
    fp.idx[q] = valid ? gy * V.st[1] + gz * V.st[2] + bb : -1;
    fp.dst[q] = idx < G::PLANE ? (bb * G::PY + yy) * G::PZ + zz : -1;
  }
}

template <class F, int TZ, int TY, int RPT>
__device__ __forceinline__ void fetch_plane(const Params& P, const View& V, const float* __restrict__ s,
                                            int64_t npad, int x, const FetchPlan<F, TZ, TY, RPT>& fp,
                                            PlaneRegs<F, TZ, TY, RPT>& pr) {
  using G = Geo<F, TZ, TY, RPT>;
  bool xvalid = true;
  const int gx = wrap_sel(x, V.L[0], V.per[0], xvalid);
  const float* sx = s + V.offset + gx * V.st[0];
#pragma unroll
  for (int q = 0; q < G::PER_THREAD; ++q) {
    const bool valid = xvalid && fp.idx[q] >= 0 &&
                       LLG_IN_RANGE(P, (int64_t)gx * V.st[0] + fp.idx[q], 0, (int64_t)V.L[0] * V.st[0]);
    const int i = fp.idx[q];
    pr.v[q][0] = valid ? __ldg(sx + i) : 0.f;
    pr.v[q][1] = valid ? __ldg(sx + npad + i) : 0.f;
    pr.v[q][2] = valid ? __ldg(sx + 2 * npad + i) : 0.f;
  }
}

template <class F, int TZ, int TY, int RPT>
__device__ __forceinline__ void store_plane(const Params& P, float4* ring, int x, const FetchPlan<F, TZ, TY, RPT>& fp,
                                            const PlaneRegs<F, TZ, TY, RPT>& pr) {
  using G = Geo<F, TZ, TY, RPT>;
  float4* slot = ring + (x & 3) * G::PLANE;
#pragma unroll
  for (int q = 0; q < G::PER_THREAD; ++q)
    if (fp.dst[q] >= 0 && LLG_IN_RANGE(P, fp.dst[q], 0, G::PLANE))
      slot[fp.dst[q]] = make_float4(pr.v[q][0], pr.v[q][1], pr.v[q][2], 0.f);
}

// ------------------------------------------------------ TMA plane fetch --
// The plane x + 2 can instead arrive by TMA: one thread issues a
// cp.async.bulk.tensor box load (the plane's rows y0 - RY .. y0 + TY + RY - 1,
// the three components as a fourth dimension) into one of two staging
// buffers, completion is counted on an mbarrier, and the threads transpose
// the box (one float per component) into the float4 ring.  Coordinates
// outside the lattice read zeros (open boundaries); positions that wrap
// around a periodic y or z boundary are read from global memory instead.
// The box starts on a 16-byte boundary: LO elements before z0 - RZ.

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// waits for phase `parity` of the mbarrier for at most about a second of
// wall time (a poll may suspend the thread for a while); false when it gave up
constexpr uint64_t kTmaWaitNs = 1000000000ull;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (global_ns() - t0 < kTmaWaitNs)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

template <class F, int TZ, int TY>
struct TmaGeo {
  static constexpr int NB = F::NB, RY = F::RY, RZ = F::RZ;
  static constexpr int LO = (RZ * NB) % 4 == 0 ? 0 : 4 - (RZ * NB) % 4;
  static constexpr int BW = ((TZ + 2 * RZ) * NB + LO + 3) / 4 * 4;   // box width, elements
  static constexpr int ROWS = TY + 2 * RY;
  static constexpr int STG = 3 * ROWS * BW;                         // floats of one box
  static constexpr int STG_PAD = (STG * 4 + 127) / 128 * 128;       // bytes of one staging buffer
  static constexpr bool FITS = BW <= 256 && ROWS <= 256;            // TMA box dimensions are at most 256
};

// per thread: the ring positions it transposes (ring order, idx = tid + q
// NT) and where each comes from: >= 0 the box offset of component 0, < 0
// -(spin index in the plane) - 1 of a periodic image read from global memory
template <class F, int TZ, int TY, int RPT>
struct TmaPlan {
  int src[Geo<F, TZ, TY, RPT>::PER_THREAD];
};

template <class F, int TZ, int TY, int RPT>
__device__ __forceinline__ void plan_tma(const View& V, int y0, int z0, int tid, TmaPlan<F, TZ, TY, RPT>& tp) {
  using G = Geo<F, TZ, TY, RPT>;
  using T = TmaGeo<F, TZ, TY>;
#pragma unroll
  for (int q = 0; q < G::PER_THREAD; ++q) {
    const int idx = tid + q * G::NT;
    const int zz = idx % G::PZ;
    const int yy = (idx / G::PZ) % G::PY;
    const int bb = idx / (G::PZ * G::PY);
    const int cy = y0 - F::RY + yy, cz = z0 - F::RZ + zz;
    const bool inside = cy >= 0 && cy < V.L[1] && cz >= 0 && cz < V.L[2];
    int src = yy * T::BW + zz * G::NB + bb + T::LO;
    if (!inside && idx < G::PLANE) {
      // a periodic image comes from global memory; a position outside an
      // open boundary keeps the box's zero
      bool valid = true;
      const int gy = wrap_sel(cy, V.L[1], V.per[1], valid);
      const int gz = wrap_sel(cz, V.L[2], V.per[2], valid);
      if (valid) src = -(gy * (int)V.st[1] + gz * (int)V.st[2] + bb) - 1;
    }
    tp.src[q] = src;
  }
}

// the box of plane x (staging buffer `stg`) into ring slot x & 3
template <class F, int TZ, int TY, int RPT>
__device__ __forceinline__ void transpose_plane(const Params& P, const View& V, const float* __restrict__ s,
                                                int x, const float* stg, float4* ring, const TmaPlan<F, TZ, TY, RPT>& tp) {
  using G = Geo<F, TZ, TY, RPT>;
  using T = TmaGeo<F, TZ, TY>;
  bool xvalid = true;
  const int gx = wrap_sel(x, V.L[0], V.per[0], xvalid);
  const float* sx = s + V.offset + (int64_t)gx * V.st[0];
  float4* slot = ring + (x & 3) * G::PLANE;
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
#pragma unroll
  for (int q = 0; q < G::PER_THREAD; ++q) {
    const int idx = tid + q * G::NT;
    if (idx < G::PLANE) {
      const int src = tp.src[q];
      float4 v;
      if (src >= 0) {
        const bool ok = LLG_IN_RANGE(P, src + 2 * T::ROWS * T::BW, 0, T::STG);
        v = ok ? make_float4(stg[src], stg[src + T::ROWS * T::BW], stg[src + 2 * T::ROWS * T::BW], 0.f)
               : make_float4(0.f, 0.f, 0.f, 0.f);
      } else {
        const int i = -src - 1;
        const bool ok = xvalid && LLG_IN_RANGE(P, (int64_t)gx * V.st[0] + i, 0, (int64_t)V.L[0] * V.st[0]);
        v = ok ? make_float4(__ldg(sx + i), __ldg(sx + P.npad + i), __ldg(sx + 2 * P.npad + i), 0.f)
               : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      slot[idx] = v;
    }
  }
}

// one thread: the box of plane x into staging buffer x & 1
template <class F, int TZ, int TY>
__device__ __forceinline__ void issue_plane(const CUtensorMap* map, const View& V, int x, int y0, int z0,
                                            unsigned char* stg_base, uint64_t* bars) {
  using T = TmaGeo<F, TZ, TY>;
  bool xvalid = true;
  const int gx = wrap_sel(x, V.L[0], V.per[0], xvalid);
  const int k = x & 1;
  // the threads' reads of this buffer (generic proxy) come before the TMA
  // write (async proxy) that overwrites it
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_expect_tx(&bars[k], (uint32_t)(T::STG * 4));
  // a plane outside an open x boundary: a plane coordinate out of range reads zeros
  tma_load_4d(stg_base + k * T::STG_PAD, map, &bars[k], (z0 - F::RZ) * F::NB - T::LO, y0 - F::RY,
              xvalid ? gx : -1, 0);
}

}  // namespace

// STAGE: 0 Heun predictor (writes sp; with aux != null also the corrector's
//          partial sum s0 + dt/2 rhs(s0) into aux)
//        1 Heun corrector recomputing rhs(s0) (rings of s0 and sp)
//        2 Heun corrector from the stored partial sum (ring of sp; own aux)
//        7 stage 0 that also writes the step's thermal field (P.noise32)
//        8 stage 2 that reads the thermal field instead of drawing it again
//          (stored-noise mode: 12 B per spin more traffic each way, no
//          second Philox draw and Box-Muller in the corrector; the same
//          values, so the same results)
//        3..6 RK4 stages 1..4 (ring of sin; own s0, aux = k accumulator)
// RPT: rows per thread.  With RPT = 2 a thread computes two neighbouring
// rows of its column in every plane, so the per-plane work of a thread
// (loop, addresses, fetch bookkeeping, barrier) is shared by two spins and
// the two rows' neighbour loads overlap; each spin's arithmetic is the same
// as with RPT = 1, so the results agree bit for bit.
// TMA: the gathered state's planes arrive by TMA box loads (tmap: the
// tensor map of the buffer the stage gathers from); one ring only, so STAGE 1
// (two rings) always stages through registers.
template <class F, int TZ, int TY, int RPT, int STG, int MINB, bool DIP, bool TMA>
__global__ void __launch_bounds__(Geo<F, TZ, TY, RPT>::NT, MINB)
    tiled_stage(const __grid_constant__ Params P, const __grid_constant__ TiledParams TP, const float* s0,
                const float* sin, float* out, float* aux, uint32_t kstep, uint32_t advance,
                const __grid_constant__ CUtensorMap tmap) {
  using G = Geo<F, TZ, TY, RPT>;
  // the stage computed; stages 7 and 8 are stages 0 and 2 that store / load
  // the thermal field
  constexpr int STAGE = STG == 7 ? 0 : (STG == 8 ? 2 : STG);
  constexpr bool WSTORE = STG == 7, WLOAD = STG == 8;
  constexpr int NR = STAGE == 1 ? 2 : 1;
  constexpr int TYT = TY / RPT;   // thread rows per basis site
  constexpr bool USE_TMA = TMA && NR == 1;
  // packed x / y neighbour sums: the two-row kernels outside the fcc
  // families (where they measured faster without costing spills)
  constexpr bool PACK = RPT == 2 && !std::is_same<F, FamFCC>::value && !std::is_same<F, FamFCC2>::value;
  static_assert(TY % RPT == 0, "rows per thread must divide the tile rows");
  static_assert(!USE_TMA || TmaGeo<F, TZ, TY>::FITS, "TMA box dimensions are at most 256");
  extern __shared__ __align__(128) float4 smem[];
  // TMA: two staging buffers on a 128-byte boundary, then the ring, then the
  // two mbarriers
  unsigned char* sbase = reinterpret_cast<unsigned char*>(smem);
  if constexpr (USE_TMA) sbase += (128u - (smem_u32(smem) & 127u)) & 127u;
  float4* ring0 = USE_TMA ? reinterpret_cast<float4*>(sbase + 2 * TmaGeo<F, TZ, TY>::STG_PAD) : smem;
  float4* ring1 = ring0 + 4 * G::PLANE;    // second ring (s0) for STAGE 1
  uint64_t* bars = reinterpret_cast<uint64_t*>(ring0 + NR * 4 * G::PLANE);
  __shared__ int s_abort;   // a TMA wait gave up: every thread leaves the plane loop
  // programmatic dependent launch: the next stage's CTAs may be scheduled
  // once every CTA of this one has started; they set up, then wait for this
  // launch to complete before they read what it wrote
  asm volatile("griddepcontrol.launch_dependents;");
  const int4 tile0 = TP.tiles[blockIdx.x];
  constexpr bool UV = RPT == 1;   // per-CTA view in uniform registers
  const int4 tile =
      make_int4(uniform<UV>(tile0.x), uniform<UV>(tile0.y), uniform<UV>(tile0.z), uniform<UV>(tile0.w));
  const ReplicaDev& R = P.rep[tile.x];
  const View V = load_view<UV>(R);
  const int thermal = uniform<UV>(R.thermal);
  const int x0 = tile.y, y0 = tile.z, z0 = tile.w;
  const int tid = threadIdx.x + TZ * threadIdx.y;
  const int tz = threadIdx.x;
  const int ty = (threadIdx.y % TYT) * RPT;   // the first of the thread's rows
  const int b = __shfl_sync(0xffffffffu, (int)(threadIdx.y / TYT), 0);   // uniform per warp
  const float amp = uniform<UV>(R.amp32[b]);
  const int z = z0 + tz;
  bool active[RPT];   // the row's cell lies in the lattice
  int own[RPT], yz[RPT];
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    const int y = y0 + ty + r;
    active[r] = y < V.L[1] && z < V.L[2];
    own[r] = (ty + r + F::RY) * G::PZ + (tz + F::RZ);
    // the stencil offsets are compile-time; they stay inside the ring slot
    // when the thread's own cell does
    if (!LLG_IN_RANGE(P, own[r], F::RY * G::PZ + F::RZ, (TY + F::RY) * G::PZ)) active[r] = false;
    yz[r] = y * V.st[1] + z * V.st[2] + b;
  }
  const float* gather_src = STAGE == 0 ? s0 : sin;
  LocalField L = local_field(P, R, b, TP.exch_term);
  constexpr bool has_dip = DIP;   // the model has a dipole term (field planes in P.hdip32)
  const float dt = P.dt32;
  // planes of this replica (outputs, stored rhs / k sum, own start state)
  float* ox = out + V.offset;
  float* oy = ox + P.npad;
  float* oz = oy + P.npad;
  float* ax = aux ? aux + V.offset : nullptr;
  float* ay = aux ? ax + P.npad : nullptr;
  float* az = aux ? ay + P.npad : nullptr;
  const float* s0x = s0 + V.offset;
  const float* s0y = s0x + P.npad;
  const float* s0z = s0y + P.npad;
  int xe = min(x0 + TP.TX, V.L[0]);
  FetchPlan<F, TZ, TY, RPT> fp;
  TmaPlan<F, TZ, TY, RPT> tp;
  if constexpr (USE_TMA) {
    plan_tma<F, TZ, TY, RPT>(V, y0, z0, tid, tp);
    if (tid == 0) {
      mbar_init(&bars[0], 1);
      mbar_init(&bars[1], 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      s_abort = 0;
    }
    __syncthreads();
  } else {
    plan_fetch<F, TZ, TY, RPT>(V, y0, z0, tid, fp);
  }
  // everything below reads the output of earlier launches (spins, stored
  // rhs, dipole field, step counter): wait for them to complete (returns at
  // once for a launch without a programmatic dependency)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const uint64_t step = uniform<UV>((unsigned long long)*P.step_base) + kstep;
  // applied-field and zeeman terms at this stage's time (Heun predictor 0,
  // corrector 1; RK4 stages 0..3) and, for the recomputed rhs(s0), at the
  // predictor's
  field_terms_hb(P, R, b, pulse_at32(P, step, STAGE == 0 ? 0 : (STAGE <= 2 ? 1 : STAGE - 3)), L.hb);
  float hb0[3] = {0.f, 0.f, 0.f};
  if (STAGE == 1) field_terms_hb(P, R, b, pulse_at32(P, step, 0), hb0);

  // TMA: planes x are waited for in order; bit k of `phase` is the parity
  // of the next completion of staging buffer k; thread 0 counts the planes it
  // issued and waited for
  uint32_t phase = 0;
  int issued = 0, waited = 0;
  auto wait_transpose = [&](int x) {
    if constexpr (USE_TMA) {
      const int k = x & 1;
      if (!mbar_wait(&bars[k], (phase >> k) & 1u)) s_abort = 1;
      phase ^= 1u << k;
      ++waited;
      transpose_plane<F, TZ, TY, RPT>(P, V, gather_src, x,
                                      reinterpret_cast<const float*>(sbase + k * TmaGeo<F, TZ, TY>::STG_PAD), ring0, tp);
    }
  };
  auto issue = [&](int x) {
    if constexpr (USE_TMA) {
      if (tid == 0) {
        issue_plane<F, TZ, TY>(&tmap, V, x, y0, z0, sbase, bars);
        ++issued;
      }
    }
  };
  if constexpr (USE_TMA) {
    issue(x0 - 1);
    issue(x0);
    wait_transpose(x0 - 1);
    wait_transpose(x0);
    __syncthreads();   // both staging buffers read
    issue(x0 + 1);
    if (x0 + 2 <= xe) issue(x0 + 2);
    wait_transpose(x0 + 1);
  } else {
    PlaneRegs<F, TZ, TY, RPT> pr;
#pragma unroll
    for (int d = -1; d <= 1; ++d) {
      fetch_plane<F, TZ, TY, RPT>(P, V, gather_src, P.npad, x0 + d, fp, pr);
      store_plane<F, TZ, TY, RPT>(P, ring0, x0 + d, fp, pr);
      if (NR == 2) {
        fetch_plane<F, TZ, TY, RPT>(P, V, s0, P.npad, x0 + d, fp, pr);
        store_plane<F, TZ, TY, RPT>(P, ring1, x0 + d, fp, pr);
      }
    }
  }
  __syncthreads();
  if constexpr (USE_TMA) {
    if (s_abort) xe = x0;   // every thread skips the plane loop
  }
  // carried partial sums of the separable stencils (ring1: s0 of STAGE 1)
  Carry cy0[RPT], cy1[RPT];
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    carry_init<F, TZ, TY>(b, ring0, x0, own[r], cy0[r]);
    if (NR == 2) carry_init<F, TZ, TY>(b, ring1, x0, own[r], cy1[r]);
  }

  // noise of plane x + 1, drawn with plane x's when x is even (the host keeps
  // planes per CTA even, so x0 is even)
  float wn[RPT][3];
#pragma unroll
  for (int r = 0; r < RPT; ++r) wn[r][0] = wn[r][1] = wn[r][2] = 0.f;
  for (int x = x0; x < xe; ++x) {
    const bool more = x + 1 < xe;
    PlaneRegs<F, TZ, TY, RPT> pf0, pf1;
    if constexpr (USE_TMA) {
      // plane x + 3 into the staging buffer plane x + 1 left (read before
      // the last barrier); plane x + 2 is already on its way
      if (x + 3 <= xe) issue(x + 3);
    } else if (more) {
      fetch_plane<F, TZ, TY, RPT>(P, V, gather_src, P.npad, x + 2, fp, pf0);
      if (NR == 2) fetch_plane<F, TZ, TY, RPT>(P, V, s0, P.npad, x + 2, fp, pf1);
    }
    // one row: skipped outside the lattice; two rows: both computed (rows
    // outside the lattice see zeros in the ring), their loads and stores
    // guarded, so that the two rows' work interleaves
    if (RPT > 1 || active[0]) {
      int ir[RPT];
      bool ldr[RPT];
      float w[RPT][3];
      // the spin's own start-of-step state, stored rhs / k sum and dipole
      // field (input state; s0 for the recomputed rhs): loaded before the
      // exchange sums so that the sums cover their latency
      float own_s0[RPT][3], own_r[RPT][3], dip[RPT][3], dip0[RPT][3];
#pragma unroll
      for (int r = 0; r < RPT; ++r) {
        const int i = x * V.st[0] + yz[r];   // spin index in the replica
        const bool ld = (RPT == 1 || active[r]) && LLG_IN_RANGE(P, i, 0, (int64_t)V.L[0] * V.st[0]);
        ir[r] = i;
        ldr[r] = ld;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          // the stored-noise predictor keeps no noise across planes: plane
          // x + 1's comes back from its store (below)
          w[r][m] = WSTORE ? 0.f : wn[r][m];
          own_s0[r][m] = own_r[r][m] = dip[r][m] = dip0[r][m] = 0.f;
        }
        if (STAGE >= 3 && ld) {
          own_s0[r][0] = __ldg(s0x + i);
          own_s0[r][1] = __ldg(s0y + i);
          own_s0[r][2] = __ldg(s0z + i);
        }
        if ((STAGE == 2 || STAGE >= 4) && ld) {
          own_r[r][0] = ax[i];
          own_r[r][1] = ay[i];
          own_r[r][2] = az[i];
        }
        if (WLOAD && ld) {   // zeros for a replica at 0 K (the host clears its planes)
#pragma unroll
          for (int m = 0; m < 3; ++m) w[r][m] = __ldg(P.noise32 + m * P.npad + V.offset + i);
        }
        if (WSTORE && ld && thermal && (x & 1)) {
          // written by this thread one plane earlier (a plain load: the
          // planes change within the launch)
#pragma unroll
          for (int m = 0; m < 3; ++m) w[r][m] = P.noise32[m * P.npad + V.offset + i];
        }
        if (has_dip && ld) {
#pragma unroll
          for (int m = 0; m < 3; ++m) dip[r][m] = __ldg(P.hdip32 + m * P.npad + V.offset + i);
          if (STAGE == 1) {
#pragma unroll
            for (int m = 0; m < 3; ++m) dip0[r][m] = __ldg(P.hdip32_s0 + m * P.npad + V.offset + i);
          }
        }
      }
      if (!WLOAD && thermal && (x & 1) == 0) {
#pragma unroll
        for (int r = 0; r < RPT; ++r)
          noise_pair(P.philox_keys, (uint32_t)tile.x, step, (uint32_t)ir[r], amp, w[r], wn[r]);
        if constexpr (WSTORE) {
          // the thermal field of planes x and x + 1 for the corrector (and
          // plane x + 1's for this thread's next plane)
#pragma unroll
          for (int r = 0; r < RPT; ++r) {
            const int i = ir[r];
            float* nz = P.noise32 + V.offset;
            if (ldr[r]) {
#pragma unroll
              for (int m = 0; m < 3; ++m) nz[m * P.npad + i] = w[r][m];
            }
            if (ldr[r] && x + 1 < xe && LLG_IN_RANGE(P, i + V.st[0], 0, (int64_t)V.L[0] * V.st[0])) {
#pragma unroll
              for (int m = 0; m < 3; ++m) nz[m * P.npad + i + V.st[0]] = wn[r][m];
            }
          }
        }
      }
#pragma unroll
      for (int r = 0; r < RPT; ++r) {
        const int i = ir[r];
        const bool st = (RPT == 1 || active[r]) && LLG_IN_RANGE(P, i, 0, (int64_t)V.L[0] * V.st[0]);
        float h[3], s[3], k[3];
        field_tiled<F, TZ, TY, PACK>(L, TP, b, ring0, x, own[r], cy0[r], h, s, has_dip, dip[r]);
        llg_rhs_t(L, s, h, w[r], k);
        if (STAGE == 0) {
          float v[3] = {ff(dt, k[0], s[0]), ff(dt, k[1], s[1]), ff(dt, k[2], s[2])};
          normalise_t(v);
          if (st) {
            ox[i] = v[0];
            oy[i] = v[1];
            oz[i] = v[2];
            if (ax) {
              // the stored-rhs corrector's partial sum s0 + dt/2 rhs(s0)
              const float hdt = fm(0.5f, dt);
              ax[i] = ff(hdt, k[0], s[0]);
              ay[i] = ff(hdt, k[1], s[1]);
              az[i] = ff(hdt, k[2], s[2]);
            }
          }
        } else if (STAGE == 1 || STAGE == 2) {
          // s1 = unit(a + dt/2 rhs(s_pred)), a = s0 + dt/2 rhs(s0): computed
          // here from the second ring (recompute) or the predictor's store
          const float hdt = fm(0.5f, dt);
          float a[3];
          if (STAGE == 1) {
            float h0[3], s0v[3], r0[3];
            LocalField L0 = L;
            L0.hb[0] = hb0[0];
            L0.hb[1] = hb0[1];
            L0.hb[2] = hb0[2];
            field_tiled<F, TZ, TY, PACK>(L0, TP, b, ring1, x, own[r], cy1[r], h0, s0v, has_dip, dip0[r]);
            llg_rhs_t(L, s0v, h0, w[r], r0);
#pragma unroll
            for (int m = 0; m < 3; ++m) a[m] = ff(hdt, r0[m], s0v[m]);
          } else {
#pragma unroll
            for (int m = 0; m < 3; ++m) a[m] = own_r[r][m];
          }
          float v[3] = {ff(hdt, k[0], a[0]), ff(hdt, k[1], a[1]), ff(hdt, k[2], a[2])};
          normalise_t(v);
          if (st) {
            if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) atomicOr(P.status, 1u);
            ox[i] = v[0];
            oy[i] = v[1];
            oz[i] = v[2];
          }
        } else {
          const float* a = own_s0[r];
          float* acc[3] = {ax, ay, az};
          float v[3];
          if (STAGE == 6) {
            const float c = fm(dt, 1.0f / 6.0f);
#pragma unroll
            for (int m = 0; m < 3; ++m) v[m] = ff(c, fa(own_r[r][m], k[m]), a[m]);
            normalise_t(v);
            if (st && !(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) atomicOr(P.status, 1u);
          } else {
            const float c = STAGE == 5 ? dt : fm(0.5f, dt);
#pragma unroll
            for (int m = 0; m < 3; ++m) {
              const float an = STAGE == 3 ? k[m] : ff(2.0f, k[m], own_r[r][m]);
              if (st) acc[m][i] = an;
              v[m] = ff(c, k[m], a[m]);
            }
            if (P.rk4_normalise_stages) normalise_t(v);
          }
          if (st) {
            ox[i] = v[0];
            oy[i] = v[1];
            oz[i] = v[2];
          }
        }
      }
    }
    if constexpr (USE_TMA) {
      if (more) wait_transpose(x + 2);
    } else if (more) {
      store_plane<F, TZ, TY, RPT>(P, ring0, x + 2, fp, pf0);
      if (NR == 2) store_plane<F, TZ, TY, RPT>(P, ring1, x + 2, fp, pf1);
    }
    __syncthreads();
    if constexpr (USE_TMA) {
      if (s_abort) break;   // read after the barrier: the same in every thread
    }
  }
  if constexpr (USE_TMA) {
    if (s_abort && tid == 0) {
      // report, and let the copies still in flight land (bounded) before the
      // CTA's shared memory is released
      atomicOr(P.status, 4u);
      for (int x = x0 - 1 + waited; waited < issued; ++x, ++waited)
        mbar_wait(&bars[x & 1], (phase >> (x & 1)) & 1u), phase ^= 1u << (x & 1);
    }
  }
  // the launch that ends a block of steps advances the noise step counter by
  // `advance`: the last CTA to finish does it, when every CTA has read the
  // counter (each read precedes its CTA's barriers and its ticket)
  if (advance != 0 && tid == 0) {
    __threadfence();
    if (atomicAdd(P.ticket, 1u) == gridDim.x - 1) {
      *P.step_base += advance;
      *P.ticket = 0u;
      __threadfence();
    }
  }
}

// ------------------------------------------------------------ launchers --

namespace {

template <class F, int TZ, int TY>
size_t smem_bytes(int stage, bool tma) {
  const size_t rings = (size_t)(stage == 1 ? 2 : 1) * 4 * Geo<F, TZ, TY>::PLANE * sizeof(float4);
  // TMA (one ring): alignment slack, two staging buffers, two mbarriers
  return tma && stage != 1 ? rings + 128 + 2 * (size_t)TmaGeo<F, TZ, TY>::STG_PAD + 16 : rings;
}

template <class F, int TZ, int TY, int RPT, int STAGE, int MINB, bool DIP, bool TMA>
cudaError_t launch_one(unsigned grid, cudaStream_t st, const Params& P, const TiledParams& TP, const float* s0,
                       const float* sin, float* out, float* aux, uint32_t k, uint32_t adv, const CUtensorMap* map) {
  if constexpr (TMA && STAGE == 1) {
    // two rings: the register-staged kernel
    return launch_one<F, TZ, TY, RPT, STAGE, MINB, DIP, false>(grid, st, P, TP, s0, sin, out, aux, k, adv, map);
  } else {
    const size_t sm = smem_bytes<F, TZ, TY>(STAGE, TMA);
    static bool attr = false;
    if (!attr) {
      cudaError_t e = cudaFuncSetAttribute(tiled_stage<F, TZ, TY, RPT, STAGE, MINB, DIP, TMA>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return e;
      attr = true;
    }
    if (TMA && !map) return cudaErrorInvalidValue;
    CUtensorMap none{};
    // launched with programmatic stream serialisation: its setup overlaps the
    // end of the previous kernel in the stream (CUDA graphs keep the
    // programmatic edge)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(TZ, (TY / RPT) * F::NB);
    cfg.dynamicSmemBytes = sm;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, tiled_stage<F, TZ, TY, RPT, STAGE, MINB, DIP, TMA>, P, TP, s0, sin, out, aux, k,
                              adv, TMA ? *map : none);
  }
}

template <class F, int TZ, int TY, int RPT, int MINB, bool DIP, bool TMA>
cudaError_t launch_family(int stage, unsigned grid, cudaStream_t st, const Params& P, const TiledParams& TP,
                          const float* s0, const float* sin, float* out, float* aux, uint32_t k, uint32_t adv,
                          const CUtensorMap* map) {
  switch (stage) {
    case 0: return launch_one<F, TZ, TY, RPT, 0, MINB, DIP, TMA>(grid, st, P, TP, s0, sin, out, aux, k, adv, map);
    case 1: return launch_one<F, TZ, TY, RPT, 1, MINB, DIP, TMA>(grid, st, P, TP, s0, sin, out, aux, k, adv, map);
    case 2: return launch_one<F, TZ, TY, RPT, 2, MINB, DIP, TMA>(grid, st, P, TP, s0, sin, out, aux, k, adv, map);
    case 3: return launch_one<F, TZ, TY, RPT, 3, MINB, DIP, TMA>(grid, st, P, TP, s0, sin, out, aux, k, adv, map);
    case 4: return launch_one<F, TZ, TY, RPT, 4, MINB, DIP, TMA>(grid, st, P, TP, s0, sin, out, aux, k, adv, map);
    case 5: return launch_one<F, TZ, TY, RPT, 5, MINB, DIP, TMA>(grid, st, P, TP, s0, sin, out, aux, k, adv, map);
    case 6: return launch_one<F, TZ, TY, RPT, 6, MINB, DIP, TMA>(grid, st, P, TP, s0, sin, out, aux, k, adv, map);
    case 7: return launch_one<F, TZ, TY, RPT, 7, MINB, DIP, TMA>(grid, st, P, TP, s0, sin, out, aux, k, adv, map);
    default: return launch_one<F, TZ, TY, RPT, 8, MINB, DIP, TMA>(grid, st, P, TP, s0, sin, out, aux, k, adv, map);
  }
}

template <class F, int TZ, int TY, int RPT, bool DIP, bool TMA>
cudaError_t launch_occ(int occupancy, int stage, unsigned grid, cudaStream_t st, const Params& P,
                       const TiledParams& TP, const float* s0, const float* sin, float* out, float* aux, uint32_t k,
                       uint32_t adv, const CUtensorMap* map) {
  // occupancy variant, as the resident threads of 2, 3 or 4 CTAs of 256
  // threads (up to 128, 80 or 64 registers per thread); CTAs of 128 threads
  // (narrow tiles, two rows per thread) run twice as many per SM with the
  // same register budget.  Two rows per thread need up to 128 registers:
  // they run at occupancy 2 only.
  constexpr int S = 256 / Geo<F, TZ, TY, RPT>::NT > 1 ? 256 / Geo<F, TZ, TY, RPT>::NT : 1;
  if constexpr (RPT == 1) {
    if (occupancy >= 4) return launch_family<F, TZ, TY, 1, 4 * S, DIP, TMA>
        (stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
    if (occupancy == 3) return launch_family<F, TZ, TY, 1, 3 * S, DIP, TMA>
        (stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
  }
  return launch_family<F, TZ, TY, RPT, 2 * S, DIP, TMA>(stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
}

}  // namespace

// the tiled stage kernels with (DIP) or without the dipole field planes, one
// (RPT = 1) or two rows per thread, planes staged through registers or by
// TMA (TMA); llg_tiled.cu instantiates <false, 1, false>, llg_tiled_dipole.cu
// <true, 1, false>, llg_tiled_pair.cu <false, 2, false>, llg_tiled_tma.cu
// <false, 1, true> and llg_tiled_tma_pair.cu <false, 2, true>.
// ty: rows of the CTA tile, the family's wide tile or, for simple cubic,
// the narrow one (half the rows: twice the CTAs, for small lattices; the
// bcc narrow tile measured slower at 64^3 and 256^3, its halo rows cost more
// than the extra CTAs gain).  Two rows per thread: the wide tiles of the
// families with at least two rows (not triangular).  TMA: the 32-cell-wide
// tiles (not triangular); map is the tensor map of the gathered buffer.
template <bool DIP, int RPT, bool TMA>
cudaError_t launch_tiled_t(int family, int ty, int occupancy, int stage, unsigned grid, cudaStream_t st,
                           const Params& P, const TiledParams& TP, const float* s0, const float* sin, float* out,
                           float* aux, uint32_t k, uint32_t adv, const CUtensorMap* map) {
  if constexpr (RPT == 1) {
    switch (family) {
      case kFamSC:
        return ty == 4 ? launch_occ<FamSC, 32, 4, 1, DIP, TMA>(occupancy, stage, grid, st, P, TP, s0, sin, out, aux,
                                                               k, adv, map)
                       : launch_occ<FamSC, 32, 8, 1, DIP, TMA>(occupancy, stage, grid, st, P, TP, s0, sin, out, aux,
                                                               k, adv, map);
      case kFamBCC: return launch_occ<FamBCC, 32, 4, 1, DIP, TMA>
          (occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
      case kFamBCC3: return launch_occ<FamBCC3, 32, 4, 1, DIP, TMA>
          (occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
      case kFamTRI:
        if constexpr (TMA) {
          return cudaErrorInvalidValue;
        } else {
          return launch_occ<FamTRI, 256, 1, 1, DIP, false>(occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k,
                                                           adv, map);
        }
      case kFamFCC: return launch_occ<FamFCC, 32, 2, 1, DIP, TMA>
          (occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
      case kFamFCC2: return launch_occ<FamFCC2, 32, 2, 1, DIP, TMA>
          (occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
      default: return cudaErrorInvalidValue;
    }
  } else {
    if (ty != 8 && family == kFamSC) return cudaErrorInvalidValue;
    switch (family) {
      case kFamSC: return launch_occ<FamSC, 32, 8, RPT, DIP, TMA>
          (occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
      case kFamBCC: return launch_occ<FamBCC, 32, 4, RPT, DIP, TMA>
          (occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
      case kFamBCC3: return launch_occ<FamBCC3, 32, 4, RPT, DIP, TMA>
          (occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
      case kFamFCC: return launch_occ<FamFCC, 32, 2, RPT, DIP, TMA>
          (occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
      case kFamFCC2: return launch_occ<FamFCC2, 32, 2, RPT, DIP, TMA>
          (occupancy, stage, grid, st, P, TP, s0, sin, out, aux, k, adv, map);
      default: return cudaErrorInvalidValue;
    }
  }
}

}  // namespace jams_llg
