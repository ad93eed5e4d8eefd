// Fused Heun step for the tiled FP32 stencil families: predictor and
// corrector of one step in a single sweep, compiled by llg_fused.cu.
//
// The two-pass stage kernels (llg_tiled.cuh) meet at a grid-wide dependency:
// the corrector of a spin needs the predictor state of its neighbours, so the
// predictor writes s_pred (and rhs(s0)) to HBM and a second launch reads it
// back.  Here one CTA computes the predictor over its tile plus a halo of one
// stencil reach in y and z (the cells of neighbouring tiles whose s_pred its
// own corrector reads) into a shared-memory ring, and runs the corrector one
// plane behind the predictor:
//
//   iteration x:  predictor at plane x + 1 (tile + halo) -> s_pred ring
//                 corrector at plane x (tile)            -> s1 in HBM
//
// s0 arrives in a four-plane ring with a halo of two reaches (the predictor
// of a halo cell needs its own neighbours).  Global memory sees s0 once (plus
// the halo, mostly from L2) and s1 once: 24 B per spin-step instead of 60-84
// B, and each spin's per-plane work (fetch bookkeeping, addresses, loop,
// barrier) is paid once per step instead of twice.  The halo cells' predictor
// is computed twice (by this CTA and by the tile that owns them); that
// redundancy is (tile + halo) / tile, about 1.4 for 32 x 8 cells.
//
// Arithmetic: every spin's predictor and corrector are the stored-rhs stage
// kernels' operations in the same order (rhs(s0) and the thermal field of a
// spin are carried in registers from its predictor to its corrector, and a
// halo cell's predictor is the owning tile's, with the same Philox noise), so
// the results equal the two-pass kernels' bit for bit.
//
// Thread layout: as the stage kernels, 32 cells along Z per warp and the basis
// site uniform per warp (TY warps per site).  The halo cells of site b are
// taken by the first HW warps of that site, one cell per lane.
#pragma once
#include "llg_tiled.cuh"

namespace jams_llg {

namespace {

template <class F, int TY>
struct FusedGeo {
  static constexpr int NB = F::NB, RY = F::RY, RZ = F::RZ, TZ = 32;
  using G0 = Geo<F, TZ + 2 * RZ, TY + 2 * RY>;   // s0 ring: two reaches of halo
  using G1 = Geo<F, TZ, TY>;                     // s_pred ring: one reach
  static constexpr int NT = TZ * TY * NB;
  static constexpr int H = G1::PY * G1::PZ - TZ * TY;    // halo cells per basis site
  static constexpr int HW = (H + 31) / 32;               // warps of halo cells per basis site
  static constexpr int PER0 = (G0::PLANE + NT - 1) / NT; // s0 positions fetched per thread
  static constexpr int SMEM = (4 * G0::PLANE + 3 * G1::PLANE) * (int)sizeof(float4);
  static_assert(HW <= TY, "the halo cells of a site need at most as many warps as the site has");
  static_assert(NT <= 1024, "at most 1024 threads per CTA");
};

// position (row, column) in the s_pred ring of halo cell k of a site: the
// reach rows above the tile, the reach columns either side of each tile
// row, the reach rows below
template <class F, int TY>
__device__ __forceinline__ void halo_position(int k, int& yy, int& zz) {
  using FG = FusedGeo<F, TY>;
  constexpr int PZ = FG::G1::PZ, RY = F::RY, RZ = F::RZ;
  constexpr int top = RY * PZ, mid = TY * 2 * RZ;
  if (k < top) {
    yy = k / PZ;
    zz = k % PZ;
  } else if (k < top + mid) {
    const int j = k - top;
    yy = RY + j / (2 * RZ);
    const int c = j % (2 * RZ);
    zz = c < RZ ? c : FG::TZ + c;
  } else {
    const int j = k - top - mid;
    yy = RY + TY + j / PZ;
    zz = j % PZ;
  }
}

// a coordinate wrapped into [0, L) along a periodic axis (any distance), or
// invalid outside an open one
__device__ __forceinline__ int wrap_any(int c, int L, bool per, bool& valid) {
  if (c >= 0 && c < L) return c;
  if (!per) {
    valid = false;
    return 0;
  }
  const int m = c % L;
  return m < 0 ? m + L : m;
}

// exchange field of basis site B at the cell `own` of a ring of geometry
// Geo<F, TZr, TYr> (planes bm, b0, bp at the cell).  Families with separable
// bcc sums (F::SEP) evaluate the block, cross and diagonal sums of all three
// planes here instead of carrying the previous plane's along x: the same
// sums in the same order as the stage kernels' carried form, so the same
// bits.
template <class F, int TZr, int TYr, int B>
__device__ __forceinline__ void exchange_ring(const TiledParams& TP, const float4* bm, const float4* b0,
                                              const float4* bp, float hi[3], float lo[3]) {
  float2 axy[F::NSHELL];
  float az[F::NSHELL];
  float r[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int g = 0; g < F::NSHELL; ++g) {
    axy[g] = make_float2(0.f, 0.f);
    az[g] = 0.f;
  }
  if constexpr (F::SEP != 0) {
    using G = Geo<F, TZr, TYr>;
    float qm[3], qn[3];
    bcc_block<F, TZr, TYr, B>(B == 0 ? bm : b0, qm);
    bcc_block<F, TZr, TYr, B>(B == 0 ? b0 : bp, qn);
    axy[0] = make_float2(fa(qm[0], qn[0]), fa(qm[1], qn[1]));
    az[0] = fa(qm[2], qn[2]);
    if constexpr (F::SEP == 2) {
      float em[3], e0[3], en[3], d0[3];
      bcc_cross<F, TZr, TYr, B>(bm, em);
      bcc_cross<F, TZr, TYr, B>(b0, e0);
      bcc_cross<F, TZr, TYr, B>(bp, en);
      bcc_diag<F, TZr, TYr, B>(b0, d0);
      const float4 sm = bm[B * G::PY * G::PZ];
      const float4 sp = bp[B * G::PY * G::PZ];
      axy[1] = make_float2(fa(fa(sm.x, sp.x), e0[0]), fa(fa(sm.y, sp.y), e0[1]));
      az[1] = fa(fa(sm.z, sp.z), e0[2]);
      axy[2] = make_float2(fa(fa(em[0], en[0]), d0[0]), fa(fa(em[1], en[1]), d0[1]));
      az[2] = fa(fa(em[2], en[2]), d0[2]);
    }
  } else {
    gather_all<F, TZr, TYr, B>(std::make_integer_sequence<int, F::Z>{}, bm, b0, bp, axy, az, r, TP);
  }
  shell_combine<F, B>(TP, axy, az, r, hi, lo);
}

// total field (meV) and the spin of the cell at `own` (site-0 plane offset)
// of a ring of geometry Geo<F, TZr, TYr>, planes bm, b0, bp
template <class F, int TZr, int TYr>
__device__ __forceinline__ void field_ring(const LocalField& L, const TiledParams& TP, int b, const float4* bm,
                                           const float4* b0, const float4* bp, float h[3], float s[3]) {
  using G = Geo<F, TZr, TYr>;
  const float4 c = b0[b * G::PY * G::PZ];
  s[0] = c.x;
  s[1] = c.y;
  s[2] = c.z;
  float hi[3], lo[3];
  if (F::NB == 1 || b == 0) {
    exchange_ring<F, TZr, TYr, 0>(TP, bm, b0, bp, hi, lo);
  } else if (b == 1) {
    exchange_ring<F, TZr, TYr, (F::NB > 1 ? 1 : 0)>(TP, bm, b0, bp, hi, lo);
  } else if (b == 2) {
    exchange_ring<F, TZr, TYr, (F::NB > 2 ? 2 : 0)>(TP, bm, b0, bp, hi, lo);
  } else {
    exchange_ring<F, TZr, TYr, (F::NB > 3 ? 3 : 0)>(TP, bm, b0, bp, hi, lo);
  }
  local_terms(L, s, hi, lo);
#pragma unroll
  for (int m = 0; m < 3; ++m) h[m] = hi[m] + lo[m];
}

// one predictor cell: where it sits in both rings and which spin it is
struct PredCell {
  int own0;      // site-0 offset in the s0 ring
  int own1;      // site-0 offset in the s_pred ring
  int yz;        // spin index within a plane of the (wrapped) cell, -1: outside an open boundary
};

// the thermal field of a predictor cell at global plane gx (noise of planes
// gx, gx + 1 drawn together when gx is even): `carry` holds the odd
// plane's half from the previous plane of the walk
__device__ __forceinline__ void cell_noise(const Params& P, uint32_t replica, uint64_t step, int gx, int st0, int yz,
                                           float amp, bool fresh, float w[3], float carry[3]) {
  if ((gx & 1) == 0) {
    noise_pair(P.philox_keys, replica, step, (uint32_t)(gx * st0 + yz), amp, w, carry);
  } else if (fresh) {
    float wa[3];
    noise_pair(P.philox_keys, replica, step, (uint32_t)((gx - 1) * st0 + yz), amp, wa, w);
  } else {
#pragma unroll
    for (int m = 0; m < 3; ++m) w[m] = carry[m];
  }
}

// predictor of one cell at local plane p (ring slots from p): s_pred into the
// s_pred ring; rhs(s0) and the thermal field returned
template <class F, int TY>
__device__ __forceinline__ void predict_cell(const Params& P, const TiledParams& TP, const LocalField& L, int b,
                                             const PredCell& c, float4* ring0, float4* ring1, int p, bool plane_ok,
                                             int gx, int st0, uint32_t replica, uint64_t step, float amp, bool thermal,
                                             bool fresh, float dt, float k[3], float w[3], float carry[3]) {
  using FG = FusedGeo<F, TY>;
  using G0 = typename FG::G0;
  using G1 = typename FG::G1;
  float v[3] = {0.f, 0.f, 0.f};
  if (plane_ok && c.yz >= 0) {
    const float4* bm = ring0 + ((p + 3) & 3) * G0::PLANE + c.own0;
    const float4* b0 = ring0 + (p & 3) * G0::PLANE + c.own0;
    const float4* bp = ring0 + ((p + 1) & 3) * G0::PLANE + c.own0;
    float h[3], s[3];
    field_ring<F, FG::TZ + 2 * F::RZ, TY + 2 * F::RY>(L, TP, b, bm, b0, bp, h, s);
    if (thermal) {
      cell_noise(P, replica, step, gx, st0, c.yz, amp, fresh, w, carry);
    } else {
      w[0] = w[1] = w[2] = 0.f;
    }
    llg_rhs_t(L, s, h, w, k);
#pragma unroll
    for (int m = 0; m < 3; ++m) v[m] = ff(dt, k[m], s[m]);
    normalise_t(v);
  } else {
    k[0] = k[1] = k[2] = 0.f;
    w[0] = w[1] = w[2] = 0.f;
  }
  const int slot = (p + 3) % 3;
  const int dst = slot * G1::PLANE + c.own1 + b * G1::PY * G1::PZ;
  if (LLG_IN_RANGE(P, dst, 0, 3 * G1::PLANE)) ring1[dst] = make_float4(v[0], v[1], v[2], 0.f);
}

// the s0 positions a thread fetches: spin index in the plane (-1: zero) and
// ring offset (-1: none)
template <class F, int TY>
struct FusedFetch {
  int idx[FusedGeo<F, TY>::PER0];
  int dst[FusedGeo<F, TY>::PER0];
};

template <class F, int TY>
__device__ __forceinline__ void fused_plan(const View& V, int y0, int z0, int tid, FusedFetch<F, TY>& fp) {
  using FG = FusedGeo<F, TY>;
  using G0 = typename FG::G0;
#pragma unroll
  for (int q = 0; q < FG::PER0; ++q) {
    const int idx = tid + q * FG::NT;
    const int bb = idx % FG::NB;
    const int t = idx / FG::NB;
    const int zz = t % G0::PZ;
    const int yy = t / G0::PZ;
    bool valid = idx < G0::PLANE;
    const int gy = wrap_any(y0 - 2 * F::RY + yy, V.L[1], V.per[1], valid);
    const int gz = wrap_any(z0 - 2 * F::RZ + zz, V.L[2], V.per[2], valid);
    fp.idx[q] = valid ? gy * V.st[1] + gz * V.st[2] + bb : -1;
    fp.dst[q] = idx < G0::PLANE ? (bb * G0::PY + yy) * G0::PZ + zz : -1;
  }
}

template <class F, int TY>
__device__ __forceinline__ void fused_fetch(const Params& P, const View& V, const float* __restrict__ s, int x,
                                            const FusedFetch<F, TY>& fp, float (&v)[FusedGeo<F, TY>::PER0][3]) {
  bool xvalid = true;
  const int gx = wrap_any(x, V.L[0], V.per[0], xvalid);
  const float* sx = s + V.offset + (int64_t)gx * V.st[0];
#pragma unroll
  for (int q = 0; q < FusedGeo<F, TY>::PER0; ++q) {
    const int i = fp.idx[q];
    const bool valid =
        xvalid && i >= 0 && LLG_IN_RANGE(P, (int64_t)gx * V.st[0] + i, 0, (int64_t)V.L[0] * V.st[0]);
    v[q][0] = valid ? __ldg(sx + i) : 0.f;
    v[q][1] = valid ? __ldg(sx + P.npad + i) : 0.f;
    v[q][2] = valid ? __ldg(sx + 2 * P.npad + i) : 0.f;
  }
}

template <class F, int TY>
__device__ __forceinline__ void fused_store(const Params& P, float4* ring0, int x, const FusedFetch<F, TY>& fp,
                                            const float (&v)[FusedGeo<F, TY>::PER0][3]) {
  using G0 = typename FusedGeo<F, TY>::G0;
  float4* slot = ring0 + (x & 3) * G0::PLANE;
#pragma unroll
  for (int q = 0; q < FusedGeo<F, TY>::PER0; ++q)
    if (fp.dst[q] >= 0 && LLG_IN_RANGE(P, fp.dst[q], 0, G0::PLANE))
      slot[fp.dst[q]] = make_float4(v[q][0], v[q][1], v[q][2], 0.f);
}

}  // namespace

// One Heun step of the tiles TP.tiles: s0 -> s1 (distinct buffers).
template <class F, int TY, int MINB>
__global__ void __launch_bounds__(FusedGeo<F, TY>::NT, MINB)
    fused_heun(const __grid_constant__ Params P, const __grid_constant__ TiledParams TP, const float* s0, float* s1,
               uint32_t kstep, uint32_t advance) {
  using FG = FusedGeo<F, TY>;
  using G0 = typename FG::G0;
  using G1 = typename FG::G1;
  constexpr int RY = F::RY, RZ = F::RZ, TZ = FG::TZ;
  extern __shared__ float4 smem[];
  float4* ring0 = smem;                    // s0, four planes
  float4* ring1 = smem + 4 * G0::PLANE;    // s_pred, three planes
  asm volatile("griddepcontrol.launch_dependents;");
  const int4 tile0 = TP.tiles[blockIdx.x];
  const int4 tile = make_int4(uniform(tile0.x), uniform(tile0.y), uniform(tile0.z), uniform(tile0.w));
  const ReplicaDev& R = P.rep[tile.x];
  const View V = load_view<true>(R);
  const int thermal = uniform(R.thermal);
  const int x0 = tile.y, y0 = tile.z, z0 = tile.w;
  const int tid = threadIdx.x + TZ * threadIdx.y;
  const int tz = threadIdx.x;
  const int wrow = __shfl_sync(0xffffffffu, (int)(threadIdx.y % TY), 0);   // warp's row within its site
  const int b = __shfl_sync(0xffffffffu, (int)(threadIdx.y / TY), 0);      // uniform per warp
  const int ty = wrow;
  const float amp = uniform(R.amp32[b]);
  const int st0 = V.st[0];

  // the thread's tile cell (corrector and predictor)
  const int y = y0 + ty, z = z0 + tz;
  PredCell core;
  core.own0 = (ty + 2 * RY) * G0::PZ + (tz + 2 * RZ);
  core.own1 = (ty + RY) * G1::PZ + (tz + RZ);
  {
    bool valid = true;
    const int gy = wrap_any(y, V.L[1], V.per[1], valid);
    const int gz = wrap_any(z, V.L[2], V.per[2], valid);
    core.yz = valid ? gy * V.st[1] + gz * V.st[2] + b : -1;
  }
  const int yz_store = y * V.st[1] + z * V.st[2] + b;
  // the thread's halo cell (first HW warps of each site)
  const bool halo_warp = wrow < FG::HW;
  const int hk = wrow * 32 + tz;
  PredCell halo;
  halo.own0 = halo.own1 = 0;
  halo.yz = -1;
  if (halo_warp && hk < FG::H) {
    int yy, zz;
    halo_position<F, TY>(hk, yy, zz);
    halo.own0 = (yy + RY) * G0::PZ + (zz + RZ);
    halo.own1 = yy * G1::PZ + zz;
    bool valid = true;
    const int gy = wrap_any(y0 - RY + yy, V.L[1], V.per[1], valid);
    const int gz = wrap_any(z0 - RZ + zz, V.L[2], V.per[2], valid);
    halo.yz = valid ? gy * V.st[1] + gz * V.st[2] + b : -1;
  }
  bool halo_cell = halo_warp && hk < FG::H;   // lanes past the last halo cell have none
  // the stencil offsets are compile-time; they stay inside the rings when a
  // cell's own position does (checked build: a miss drops the cell; every
  // thread still reaches every barrier)
  bool active = y < V.L[1] && z < V.L[2];
  if (!LLG_IN_RANGE(P, core.own0, 2 * RY * G0::PZ + 2 * RZ, (TY + 2 * RY) * G0::PZ - 2 * RZ) ||
      !LLG_IN_RANGE(P, core.own1, RY * G1::PZ + RZ, (TY + RY) * G1::PZ - RZ)) {
    core.yz = -1;
    active = false;
  }
  if (halo_cell && (!LLG_IN_RANGE(P, halo.own0, RY * G0::PZ + RZ, (TY + 3 * RY) * G0::PZ - RZ) ||
                    !LLG_IN_RANGE(P, halo.own1, 0, G1::PY * G1::PZ)))
    halo_cell = false;
  LocalField L = local_field(P, R, b, TP.exch_term);
  const float dt = P.dt32;
  float* ox = s1 + V.offset;
  float* oy = ox + P.npad;
  float* oz = oy + P.npad;
  const int xe = min(x0 + TP.TX, V.L[0]);
  FusedFetch<F, TY> fp;
  fused_plan<F, TY>(V, y0, z0, tid, fp);

  asm volatile("griddepcontrol.wait;" ::: "memory");
  const uint64_t step = uniform((unsigned long long)*P.step_base) + kstep;
  // applied-field and zeeman terms at the predictor's and the corrector's
  // time; L.hb holds the one of the stage being computed
  float hbp[3], hbc[3];
  field_terms_hb(P, R, b, pulse_at32(P, step, 0), hbp);
  field_terms_hb(P, R, b, pulse_at32(P, step, 1), hbc);

  float reg[FG::PER0][3];
  // s0 planes x0 - 2 .. x0 + 1
#pragma unroll 1
  for (int d = -2; d <= 1; ++d) {
    fused_fetch<F, TY>(P, V, s0, x0 + d, fp, reg);
    fused_store<F, TY>(P, ring0, x0 + d, fp, reg);
  }
  __syncthreads();

  // predictor of local plane p for the tile cell (returns its rhs(s0) and
  // thermal field) and the halo cell
  float wcar[3] = {0.f, 0.f, 0.f}, hcar[3] = {0.f, 0.f, 0.f};
  auto predict = [&](int p, bool fresh, float k[3], float w[3]) {
    bool pv = true;
    const int gx = wrap_any(p, V.L[0], V.per[0], pv);
#pragma unroll
    for (int m = 0; m < 3; ++m) L.hb[m] = hbp[m];
    predict_cell<F, TY>(P, TP, L, b, core, ring0, ring1, p, pv, gx, st0, (uint32_t)tile.x, step, amp,
                        thermal != 0, fresh, dt, k, w, wcar);
    if (halo_cell) {
      float hkr[3], hw[3];
      predict_cell<F, TY>(P, TP, L, b, halo, ring0, ring1, p, pv, gx, st0, (uint32_t)tile.x, step, amp,
                          thermal != 0, fresh, dt, hkr, hw, hcar);
    }
  };

  float rhs0[3], w0[3];
  {
    float kk[3], ww[3];
    predict(x0 - 1, true, kk, ww);
  }
  __syncthreads();   // s0 of plane x0 - 2 is no longer read: its slot takes plane x0 + 2
  fused_fetch<F, TY>(P, V, s0, x0 + 2, fp, reg);
  fused_store<F, TY>(P, ring0, x0 + 2, fp, reg);
  predict(x0, false, rhs0, w0);
  __syncthreads();

#pragma unroll 1
  for (int x = x0; x < xe; ++x) {
    const bool more = x + 1 < xe;   // the predictor of plane x + 2 will run: fetch s0 of plane x + 3
    if (more) fused_fetch<F, TY>(P, V, s0, x + 3, fp, reg);
    float rhs1[3], w1[3];
    predict(x + 1, false, rhs1, w1);
    if (more) fused_store<F, TY>(P, ring0, x + 3, fp, reg);
    __syncthreads();
    // corrector of plane x
    if (active) {
      const int i = x * st0 + yz_store;
      const float4* bm = ring1 + ((x + 2) % 3) * G1::PLANE + core.own1;
      const float4* b0 = ring1 + (x % 3) * G1::PLANE + core.own1;
      const float4* bp = ring1 + ((x + 1) % 3) * G1::PLANE + core.own1;
      float h[3], s[3], k[3];
#pragma unroll
      for (int m = 0; m < 3; ++m) L.hb[m] = hbc[m];
      field_ring<F, TZ, TY>(L, TP, b, bm, b0, bp, h, s);
      llg_rhs_t(L, s, h, w0, k);
      const float4 a4 = ring0[(x & 3) * G0::PLANE + core.own0 + b * G0::PY * G0::PZ];
      const float a[3] = {a4.x, a4.y, a4.z};
      // s1 = unit(a + dt/2 rhs(s_pred)), a = s0 + dt/2 rhs(s0): the
      // stored-rhs stage kernels' operations
      const float hdt = fm(0.5f, dt);
      const float ap[3] = {ff(hdt, rhs0[0], a[0]), ff(hdt, rhs0[1], a[1]), ff(hdt, rhs0[2], a[2])};
      float v[3] = {ff(hdt, k[0], ap[0]), ff(hdt, k[1], ap[1]), ff(hdt, k[2], ap[2])};
      normalise_t(v);
      if (LLG_IN_RANGE(P, i, 0, (int64_t)V.L[0] * st0)) {
        if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) atomicOr(P.status, 1u);
        ox[i] = v[0];
        oy[i] = v[1];
        oz[i] = v[2];
      }
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      rhs0[m] = rhs1[m];
      w0[m] = w1[m];
    }
    __syncthreads();
  }
  // the launch that ends a block of steps advances the noise step counter by
  // `advance` (as the stage kernels do)
  if (advance != 0 && tid == 0) {
    __threadfence();
    if (atomicAdd(P.ticket, 1u) == gridDim.x - 1) {
      *P.step_base += advance;
      *P.ticket = 0u;
      __threadfence();
    }
  }
}

}  // namespace jams_llg

namespace jams_llg {

namespace {

template <class F, int TY, int MINB>
cudaError_t launch_fused_one(unsigned grid, cudaStream_t st, const Params& P, const TiledParams& TP, const float* s0,
                             float* s1, uint32_t k, uint32_t adv) {
  using FG = FusedGeo<F, TY>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(fused_heun<F, TY, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         FG::SMEM);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  // programmatic stream serialisation, as the stage kernels: the CTAs of the
  // next step set up while this one drains
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(FG::TZ, TY * F::NB);
  cfg.dynamicSmemBytes = FG::SMEM;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fused_heun<F, TY, MINB>, P, TP, s0, s1, k, adv);
}

// occupancy variant as resident threads per SM (2 or 4 x 256)
template <class F, int TY>
cudaError_t launch_fused_occ(int occupancy, unsigned grid, cudaStream_t st, const Params& P, const TiledParams& TP,
                             const float* s0, float* s1, uint32_t k, uint32_t adv) {
  constexpr int NT = FusedGeo<F, TY>::NT;
  constexpr int M2 = 512 / NT > 1 ? 512 / NT : 1;
  constexpr int M4 = 1024 / NT > 1 ? 1024 / NT : 1;
  if (occupancy >= 4 && M4 != M2) return launch_fused_one<F, TY, M4>(grid, st, P, TP, s0, s1, k, adv);
  return launch_fused_one<F, TY, M2>(grid, st, P, TP, s0, s1, k, adv);
}

}  // namespace

}  // namespace jams_llg
