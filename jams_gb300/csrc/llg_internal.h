// Internal device-side description of an LLG problem for the sm_103a kernels.
//
// Layout in HBM (one allocation per array, 256-byte aligned):
//   spins   structure of arrays: x plane, y plane, z plane of `npad` reals
//           each; replicas are concatenated inside every plane, replica r
//           starting at rep[r].offset (a multiple of 64 spins).  Spin order
//           inside a replica is the reference's site order
//           ((i*L2 + j)*L3 + k)*nb + m.
//   stencil per replica and exchange term, for every basis site b and
//           boundary class q: the int32 offsets j - i of the neighbours.
//           A boundary class fixes, along each axis, whether and how the
//           stencil wraps (interior cells share one class), so one small
//           table replaces a CSR matrix of 12 B per stored value.
#pragma once

#include <cstdint>

namespace jams_llg {

constexpr int kMaxBasis = 4;
constexpr int kMaxTerms = 8;
constexpr int kMaxExchange = 4;
constexpr int kMaxGroups = 12;     // isotropic shells per basis site and term
constexpr int kMaxSlots = 96;      // neighbour slots per basis site and term
constexpr int kBlock = 256;        // threads per CTA, one spin per thread
constexpr int32_t kMissing = INT32_MIN;  // neighbour outside an open boundary

enum TermKind { kExchange = 0, kUniaxial = 1, kCubic = 2, kAppliedField = 3, kDipole = 4, kZeeman = 5 };

// Bounds-checked build (compiled with LLG_BOUNDS_CHECK, a library of its own):
// every gathered or stored index is checked against its array; an index
// outside sets status bit 1, the access is skipped and llg_synchronize
// reports LLG_ERR_BOUNDS.  Nothing asserts or traps.  In the normal build
// the check is compiled out.
#ifdef LLG_BOUNDS_CHECK
#define LLG_IN_RANGE(P, j, lo, hi) \
  (((int64_t)(j) >= (int64_t)(lo) && (int64_t)(j) < (int64_t)(hi)) ? true : (atomicOr((P).status, 2u), false))
#else
#define LLG_IN_RANGE(P, j, lo, hi) true
#endif

// time factors of the time-dependent fields at one stage time t: the
// applied-field pulse's sinc and cos factors (1 when absent) and, per basis
// site, the zeeman term's cos(w_b t)
constexpr int kPulseVals = 2 + kMaxBasis;

// per exchange term, FP32 form: isotropic parts grouped into shells
// (sum of neighbour spins times one J), anisotropic remainders per slot
struct ExchangeF32 {
  int nslot[kMaxBasis];                 // slots per basis site (iso + rest)
  int ngroup[kMaxBasis];
  int group_end[kMaxBasis][kMaxGroups]; // slot index one past each group
  float group_j_hi[kMaxBasis][kMaxGroups];
  float group_j_lo[kMaxBasis][kMaxGroups];
  int nrest[kMaxBasis];                 // slots [group_end[last], nslot)
  const float* rest_j;                  // [nb][kMaxSlots][9]
};

// per exchange term, FP64 form: entries of each (b, class) in ascending
// neighbour index with the tensor and its nonzero mask
struct ExchangeF64 {
  const double* J;        // [n_entries][9]
  const uint16_t* mask;   // [n_entries] bit 3m+n set when J[m][n] != 0
};

struct TermDev {
  int kind;
  int order;              // uniaxial power, cubic order; zeeman: 1 with an ac field
  int exch;               // index into the exchange tables
  double K[kMaxBasis];
  double axis[kMaxBasis][9];  // zeeman: mu_s B_dc (0..2) and mu_s B_ac (3..5)
  float Kf[kMaxBasis];
  float axisf[kMaxBasis][9];
};

struct ReplicaDev {
  int64_t offset;         // first spin of the replica in every plane
  int32_t n;              // spins of the replica
  int32_t L[3];
  int32_t ncls[3];        // boundary classes per axis
  int32_t R[3];           // stencil reach per axis
  int32_t thermal;        // T > 0
  // table bases (element offsets) per exchange term
  int64_t tab32[kMaxExchange];   // int32 offsets [nb][ncls][nslot_max]
  int64_t tab64[kMaxExchange];   // int2 (offset, entry) [nb][ncls][zmax]
  int64_t cnt64[kMaxExchange];   // int32 counts [nb][ncls]
  double sqrt_t;          // sqrt(T)
  float amp32[kMaxBasis]; // (float)(sigma_b sqrt(T))
  double B[3];            // applied field (T)
  float Bf[3];
  // tile view for the tiled kernels: extents, spin-index strides and
  // periodicity along (X, Y, Z); Z is the contiguous axis
  int32_t vL[3];
  int64_t vs[3];
  int32_t vper[3];
};

// runtime data of the tiled FP32 kernels (llg_tiled.cuh)
struct TiledParams {
  const int4* tiles;      // (replica, x0, y0, z0) per CTA
  int ntiles;
  int TX;                 // planes streamed per CTA
  int exch_term;          // term handled by the tiled exchange
  float shell_hi[kMaxBasis][4];
  float shell_lo[kMaxBasis][4];
  float rest[kMaxBasis][8][9];
};

struct Params {
  int nb;
  int nterms;
  int nexch;
  int nslot_max[kMaxExchange];
  int zmax[kMaxExchange];
  TermDev term[kMaxTerms];
  ExchangeF32 ex32[kMaxExchange];
  ExchangeF64 ex64[kMaxExchange];
  const int32_t* tab32;   // all int32 slot tables
  const int2* tab64;      // all sorted (offset, entry) tables
  const int32_t* cnt64;
  const ReplicaDev* rep;
  const int2* tiles;      // (replica, first spin) per CTA
  int ntiles;
  int64_t npad;           // plane stride
  // per basis site material constants
  double mus[kMaxBasis];
  double gyro[kMaxBasis];
  double alpha[kMaxBasis];
  double sigma[kMaxBasis];
  float inv_mus32[kMaxBasis];
  float mus32[kMaxBasis];
  float gyro32[kMaxBasis];
  float alpha32[kMaxBasis];
  double dt;
  float dt32;
  uint64_t seed;
  int rk4_normalise_stages;
  unsigned int* status;   // bit 0: non-finite spin
  uint64_t* step_base;        // iteration number of step 0 of a launch block
  unsigned int* ticket;       // CTAs finished in the launch that advances step_base
  uint32_t philox_keys[20];   // Philox4x32-10 round keys of the seed
  // dipole field planes (meV, three planes of npad) of the stage's input
  // state and of the start-of-step state; null without a dipole term
  const float* hdip32;
  const float* hdip32_s0;
  const double* hdip64;
  const double* hdip64_s0;
  // the thermal field planes of the step (T, three planes of npad): written
  // by the tiled Heun predictor and read by the stored-rhs corrector in
  // stored-noise mode; null otherwise
  float* noise32;
  // time-dependent fields (null without): kPulseVals factors per stage of
  // every step from iteration *pulse_base on, [step][stage][kPulseVals], and
  // the factors at the current solver time for fields and energies
  const double* pulse64;
  const float* pulse32;
  const uint64_t* pulse_base;
  int pulse_stages;
  const double* pulse_now64;
  const float* pulse_now32;
};

// the time factors of stage `stage` of iteration `step`, or null (no
// time-dependent field: pulse factors 1)
__device__ __forceinline__ const double* pulse_at64(const Params& P, uint64_t step, int stage) {
  return P.pulse64 ? P.pulse64 + ((int64_t)(step - *P.pulse_base) * P.pulse_stages + stage) * kPulseVals : nullptr;
}
__device__ __forceinline__ const float* pulse_at32(const Params& P, uint64_t step, int stage) {
  return P.pulse32 ? P.pulse32 + ((int64_t)(step - *P.pulse_base) * P.pulse_stages + stage) * kPulseVals : nullptr;
}

// the dipole planes of the input state in the precision Real
template <class Real>
__device__ __forceinline__ const Real* dipole_planes(const Params& P);
template <>
__device__ __forceinline__ const float* dipole_planes<float>(const Params& P) { return P.hdip32; }
template <>
__device__ __forceinline__ const double* dipole_planes<double>(const Params& P) { return P.hdip64; }

}  // namespace jams_llg
