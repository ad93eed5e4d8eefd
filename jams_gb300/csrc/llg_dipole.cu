// Dipole-dipole field by FFT convolution: the "dipole-fft" Hamiltonian of the
// reference (src/jams/hamiltonian/cuda_dipole_fft.cu:19-343, CPU twin
// src/jams/hamiltonian/dipole_fft.cc), on the library's SoA spin planes.
//
// Per replica and basis pair (i, j) the real-space tensor
//   G_ij(e) = mu0 / (4 pi a^3) (3 r r - r^2 I) / |r|^5,  r = (e + f_i - f_j) A,
// for every cell offset e with |r| <= r_cutoff + tolerance (self term
// excluded, minimum image along periodic axes) is placed on an FFT grid of
// M = L cells along periodic axes and 2L along open ones (zero padding turns
// the circular convolution into the open-boundary sum; an open axis of one
// cell needs none) and transformed once (D2Z).  A field evaluation is then
//   scatter the spins onto the grid -> R2C -> h_i(q) = sum_j mu_j W_ij(q) S_j(q)
//   -> C2R -> h_i = mu_i h_i(r) / prod(M) back into SoA planes,
// the reference's sequence (cuda_dipole_fft.cu:184-209) with the tensor
// normalised by the grid size as there.  The transforms are this library's
// own (llg_fft.cuh): one pass per axis, the scatter fused into the first
// (real) pass and the gather into the last.  FP32C evaluates in single
// precision (float tensors computed in double); FP64 in double.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <utility>
#include <vector>

#include "llg_dipole.h"
#include "llg_fft.cuh"
#include "llg_fft_reg.cuh"

namespace jams_llg {

namespace {

constexpr double kPiD = 3.14159265358979323846;
constexpr double kJoule2meVD = 6.24150907e21;          // src/jams/helpers/consts.h:35
constexpr int kDipBlock = 256;

struct MusArr {
  double v[kMaxBasis];
};

template <class T>
struct Dev {
  T* p = nullptr;
  size_t n = 0;
  ~Dev() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    n = count;
    return count ? cudaMalloc((void**)&p, count * sizeof(T)) : cudaSuccess;
  }
};

// ------------------------------------------------------------------ kernels

// The cells of one replica's FFT grid: grid index g = o * M_h + p for point
// p of line o along the real axis h (the axes after h have one cell), split
// into (x, y, z) by two divisions; field f = component * nb + basis site.
// Along h consecutive cells are nb spins apart, so a line is also a base
// index and its L_h lattice points (the rest of the line is padding).
struct GridCells {
  int L[3], M[3];
  FastDiv dM1, dM2, dnb;
  int nb, h;
  int64_t npad, offset;
  // spin-plane index of field f at grid cell g, or -1 for a padding cell
  __device__ __forceinline__ int64_t plane_index(int f, int g) const {
    const int t = (int)fdiv((uint32_t)g, dM2);
    const int z = g - t * M[2];
    const int x = (int)fdiv((uint32_t)t, dM1);
    const int y = t - x * M[1];
    if (x >= L[0] || y >= L[1] || z >= L[2]) return -1;
    const int m = (int)fdiv((uint32_t)f, dnb), b = f - m * nb;
    return m * npad + offset + (((int64_t)x * L[1] + y) * L[2] + z) * nb + b;
  }
  // spin-plane index of point 0 of line o of field f, or -1 when the line
  // lies in the padding
  __device__ __forceinline__ int64_t line_base(int f, int o) const {
    return plane_index(f, o * M[h]);
  }
};

// the spins of one replica on its FFT grid, read by the forward real pass
// (the scatter fused into it); cells outside the lattice (padding) are zero
template <class Real>
struct SpinSource {
  const Real* s;
  GridCells gc;
  int Mh;
  __device__ Real operator()(int f, int o, int p) const {
    const int64_t i = gc.plane_index(f, o * Mh + p);
    return i < 0 ? Real(0) : __ldg(s + i);
  }
  // one line: point p is line(...)[p * nb] for p < L_h, zero beyond
  __device__ const Real* line(int f, int o) const {
    const int64_t i = gc.line_base(f, o);
    return i < 0 ? nullptr : s + i;
  }
  __device__ int length() const { return gc.L[gc.h]; }
  __device__ int step() const { return gc.nb; }
};

// a real grid of fields (the tensors at set-up)
struct GridSource {
  const double* g;
  int64_t Mtot;
  int Mh;
  __device__ double operator()(int f, int o, int p) const { return g[f * Mtot + (int64_t)o * Mh + p]; }
};

// the field planes of one replica, written by the inverse real pass (the
// gather fused into it): mu_s times the transform, lattice cells only
template <class Real>
struct FieldSink {
  Real* hp;
  GridCells gc;
  int Mh;
  MusArr mus;
  __device__ void operator()(int f, int o, int p, Real v) const {
    const int64_t i = gc.plane_index(f, o * Mh + p);
    if (i >= 0) hp[i] = (Real)mus.v[f - (int)fdiv((uint32_t)f, gc.dnb) * gc.nb] * v;
  }
  // one line (as SpinSource::line) and the moment of field f's site
  __device__ Real* line(int f, int o) const {
    const int64_t i = gc.line_base(f, o);
    return i < 0 ? nullptr : hp + i;
  }
  __device__ Real moment(int f) const { return (Real)mus.v[f - (int)fdiv((uint32_t)f, gc.dnb) * gc.nb]; }
  __device__ int length() const { return gc.L[gc.h]; }
  __device__ int step() const { return gc.nb; }
};

// h_i(q) = sum_j mu_j W_ij(q) S_j(q) for every k-space point q.  W_ij is the
// transform of a real tensor, so W_ji = conj(W_ij); W_ii is the transform of
// a tensor even in the offset, so it is real.  Stored: wd, the six real
// components (xx, xy, xz, yy, yz, zz) of every W_ii; wo, the six complex
// components of every W_ij with i < j (pair index p in row order).
template <class C>
__device__ __forceinline__ void cmac_sym(C h[3], const C g[6], const C s[3], bool conj) {
  // h += g s with g the symmetric 3x3 of six complex components (conj: of g*)
  const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
#pragma unroll
  for (int m = 0; m < 3; ++m)
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      const C a = g[idx[m][n]];
      const auto ai = conj ? -a.y : a.y;
      h[m].x += a.x * s[n].x - ai * s[n].y;
      h[m].y += a.x * s[n].y + ai * s[n].x;
    }
}

template <class C, class Real, int NB>
__global__ void __launch_bounds__(kDipBlock) dip_convolve(const C* __restrict__ ks, const Real* __restrict__ wd,
                                                          const C* __restrict__ wo, C* __restrict__ kh, int64_t Mq,
                                                          MusArr mus) {
  // programmatic dependent launch: the next pass may be scheduled now; wait
  // for the forward transform before reading its spectrum
  asm volatile("griddepcontrol.launch_dependents;");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= Mq) return;
  C s[NB][3], h[NB][3];
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const C v = ks[(int64_t)(m * NB + j) * Mq + q];
      s[j][m].x = v.x * (Real)mus.v[j];
      s[j][m].y = v.y * (Real)mus.v[j];
      h[j][m].x = h[j][m].y = 0;
    }
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    C g[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      g[c].x = wd[(int64_t)(i * 6 + c) * Mq + q];
      g[c].y = 0;
    }
    cmac_sym(h[i], g, s[i], false);
  }
  int p = 0;
#pragma unroll
  for (int i = 0; i < NB; ++i)
#pragma unroll
    for (int j = i + 1; j < NB; ++j, ++p) {
      C g[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) g[c] = wo[(int64_t)(p * 6 + c) * Mq + q];
      cmac_sym(h[i], g, s[j], false);
      cmac_sym(h[j], g, s[i], true);
    }
#pragma unroll
  for (int i = 0; i < NB; ++i)
#pragma unroll
    for (int m = 0; m < 3; ++m) kh[(int64_t)(m * NB + i) * Mq + q] = h[i][m];
}

template <class C, class Real>
cudaError_t launch_convolve(int nb, const C* ks, const Real* wd, const C* wo, C* kh, int64_t Mq, const MusArr& mus,
                            cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)((Mq + kDipBlock - 1) / kDipBlock));
  cfg.blockDim = dim3(kDipBlock);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  switch (nb) {
    case 1: return cudaLaunchKernelEx(&cfg, dip_convolve<C, Real, 1>, ks, wd, wo, kh, Mq, mus);
    case 2: return cudaLaunchKernelEx(&cfg, dip_convolve<C, Real, 2>, ks, wd, wo, kh, Mq, mus);
    case 3: return cudaLaunchKernelEx(&cfg, dip_convolve<C, Real, 3>, ks, wd, wo, kh, Mq, mus);
    default: return cudaLaunchKernelEx(&cfg, dip_convolve<C, Real, 4>, ks, wd, wo, kh, Mq, mus);
  }
}

__global__ void dip_tensor_scatter(const int64_t* __restrict__ idx, const double* __restrict__ vals, int64_t n,
                                   int64_t Mtot, double* __restrict__ grid) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  for (int c = 0; c < 6; ++c) grid[c * Mtot + idx[e]] = vals[6 * e + c];
}

// k-space tensor of one basis pair into its stored form: real parts (a
// diagonal pair) or the complex values, in the replica's precision
template <class C, class Real>
__global__ void dip_store_tensor(const double2* __restrict__ a, Real* __restrict__ real_out, C* __restrict__ cplx_out,
                                 int64_t n) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  if (real_out) {
    real_out[e] = (Real)a[e].x;
  } else {
    C v;
    v.x = (Real)a[e].x;
    v.y = (Real)a[e].y;
    cplx_out[e] = v;
  }
}

unsigned blocks(int64_t n) { return (unsigned)((n + kDipBlock - 1) / kDipBlock); }

}  // namespace

double dipole_max_radius(const double A[9], const int L[3], const int periodic[3]) {
  double v[3][3];
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 3; ++c) v[k][c] = L[k] * A[3 * k + c];
  auto cross_norm = [](const double* a, const double* b) {
    const double c0 = a[1] * b[2] - a[2] * b[1], c1 = a[2] * b[0] - a[0] * b[2], c2 = a[0] * b[1] - a[1] * b[0];
    return std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  };
  auto norm = [](const double* a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); };
  const int np = (periodic[0] != 0) + (periodic[1] != 0) + (periodic[2] != 0);
  if (np == 3) {   // inradius of the parallelepiped
    const double c0 = v[1][1] * v[2][2] - v[1][2] * v[2][1], c1 = v[1][2] * v[2][0] - v[1][0] * v[2][2],
                 c2 = v[1][0] * v[2][1] - v[1][1] * v[2][0];
    const double vol = std::fabs(v[0][0] * c0 + v[0][1] * c1 + v[0][2] * c2);
    const double h = std::min(vol / cross_norm(v[1], v[2]),
                              std::min(vol / cross_norm(v[2], v[0]), vol / cross_norm(v[0], v[1])));
    return 0.5 * h;
  }
  if (np == 2) {   // inradius of the periodic parallelogram
    const double* a = periodic[0] ? v[0] : v[1];
    const double* b = periodic[2] ? v[2] : v[1];
    const double area = cross_norm(a, b);
    return 0.5 * std::min(area / norm(a), area / norm(b));
  }
  if (np == 1) return 0.5 * norm(periodic[0] ? v[0] : (periodic[1] ? v[1] : v[2]));
  const double d[3] = {v[0][0] + v[1][0] + v[2][0], v[0][1] + v[1][1] + v[2][1], v[0][2] + v[1][2] + v[2][2]};
  return norm(d);
}

struct DipoleReplica {
  int L[3] = {1, 1, 1};
  int M[3] = {1, 1, 1};
  int64_t offset = 0;
  int64_t Mtot = 0, Mq = 0;
  int h = 2;                        // the halved (real) axis: the last one longer than one cell
  FftPlan1D plan[3] = {};
  Dev<double2> twd[3];              // W_M^t = exp(-2 pi i t / M) per axis
  Dev<float2> twf[3];
  Dev<unsigned char> ks, kh, wd, wo;   // wd: diagonal tensors (real), wo: i < j (complex)
};

struct DipoleField {
  bool fp64 = false;
  int nb = 1;
  MusArr mus{};
  std::vector<DipoleReplica*> reps;
  ~DipoleField() {
    for (auto* r : reps) delete r;
  }
};

namespace {

// --------------------------------------------------------- FFT driving --

// complex values per shared-memory buffer of a transform pass (more when
// one line is longer), and lines per CTA of a strided pass (16 x 8 B or
// 8 x 16 B: one 128-byte run of global memory per line element)
template <class C>
constexpr int fft_elems() {
  return sizeof(C) == sizeof(float2) ? 2048 : 1024;
}
template <class C>
constexpr int fft_pass_lines() {
  return sizeof(C) == sizeof(float2) ? 16 : 8;
}
inline int lines_per_cta(int n, int elems, int cap) { return std::max(1, std::min(cap, elems / n)); }

// dynamic shared memory above the default for a transform kernel (once per
// kernel and size)
cudaError_t allow_smem(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::vector<std::pair<const void*, size_t>> have;
  if (bytes <= 48 * 1024) return cudaSuccess;
  std::lock_guard<std::mutex> lock(mu);
  for (auto& e : have)
    if (e.first == kernel && e.second >= bytes) return cudaSuccess;
  const cudaError_t ce = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (ce == cudaSuccess) have.push_back({kernel, bytes});
  else cudaGetLastError();   // returned here: not left for a later check to find
  return ce;
}

template <class C>
const C* twiddles(const DipoleReplica& R, int a);
template <>
const float2* twiddles<float2>(const DipoleReplica& R, int a) {
  return R.twf[a].p;
}
template <>
const double2* twiddles<double2>(const DipoleReplica& R, int a) {
  return R.twd[a].p;
}

// length of axis b in the half-spectrum grid
int64_t kdim(const DipoleReplica& R, int b) {
  return b == R.h ? R.M[b] / 2 + 1 : (b < R.h ? R.M[b] : 1);
}

// a transform kernel on stream st; with programmatic stream serialisation
// (pdl) its twiddle load overlaps the previous kernel's tail
template <class... P, class... A>
cudaError_t launch_fft(void (*kernel)(P...), unsigned grid, size_t smem, cudaStream_t st, bool pdl, A&&... args) {
  cudaError_t ce = allow_smem((const void*)kernel, smem);
  if (ce != cudaSuccess) return ce;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kFftThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

// the register passes take single-precision lines of a power-of-two length
// in [16, 1024]
inline bool reg_length(int n) { return n >= kFftRegMin && n <= kFftRegMax && (n & (n - 1)) == 0; }

template <int N>
cudaError_t reg_pass(float2* k, int stride, int64_t outer, const float2* tw, bool inverse, cudaStream_t st,
                     bool pdl) {
  constexpr int G = 256 / RegShape<N>::T;
  const int64_t chunks = (stride + G - 1) / G;
  const unsigned grid = (unsigned)(outer * chunks);
  return inverse ? launch_fft(fft_pass_reg<N, true>, grid, reg_pass_smem<N>(), st, pdl, k, stride,
                              fast_div((uint32_t)chunks), tw)
                 : launch_fft(fft_pass_reg<N, false>, grid, reg_pass_smem<N>(), st, pdl, k, stride,
                              fast_div((uint32_t)chunks), tw);
}

// sites: the line pairs are basis-site pairs (an even number of fields,
// 8-byte aligned pairs in the planes)
template <int N, class Src>
cudaError_t reg_forward(const Src& src, int nlines, int O, bool sites, const float2* tw, float2* k, cudaStream_t st,
                        bool pdl) {
  constexpr int G = 256 / RegShape<N>::T;
  const int npairs = sites ? nlines / 2 : (nlines + 1) / 2;
  const unsigned grid = (unsigned)((npairs + G - 1) / G);
  return sites ? launch_fft(fft_real_forward_reg<N, true, Src>, grid, reg_real_smem<N>(), st, pdl, src, nlines,
                            npairs, fast_div((uint32_t)O), tw, k)
               : launch_fft(fft_real_forward_reg<N, false, Src>, grid, reg_real_smem<N>(), st, pdl, src, nlines,
                            npairs, fast_div((uint32_t)O), tw, k);
}

template <int N, class Sink>
cudaError_t reg_inverse(const float2* k, int nlines, int O, bool sites, const float2* tw, const Sink& sink,
                        cudaStream_t st, bool pdl) {
  constexpr int G = 256 / RegShape<N>::T;
  const int npairs = sites ? nlines / 2 : (nlines + 1) / 2;
  const unsigned grid = (unsigned)((npairs + G - 1) / G);
  return sites ? launch_fft(fft_real_inverse_reg<N, true, Sink>, grid, reg_real_smem<N>(), st, pdl, k, nlines,
                            npairs, fast_div((uint32_t)O), tw, sink)
               : launch_fft(fft_real_inverse_reg<N, false, Sink>, grid, reg_real_smem<N>(), st, pdl, k, nlines,
                            npairs, fast_div((uint32_t)O), tw, sink);
}

// F<N>::run(args...) for the register length n
#define JAMS_FFT_REG_SWITCH(n, CALL) \
  switch (n) {                       \
    case 16: return CALL(16);        \
    case 32: return CALL(32);        \
    case 64: return CALL(64);        \
    case 128: return CALL(128);      \
    case 256: return CALL(256);      \
    case 512: return CALL(512);      \
    default: return CALL(1024);      \
  }

template <class C>
cudaError_t reg_pass_any(int n, C* k, int stride, int64_t outer, const C* tw, bool inverse, cudaStream_t st, bool pdl) {
  if constexpr (std::is_same<C, float2>::value) {
#define JAMS_CALL(N) reg_pass<N>(k, stride, outer, tw, inverse, st, pdl)
    JAMS_FFT_REG_SWITCH(n, JAMS_CALL)
#undef JAMS_CALL
  }
  return cudaErrorInvalidValue;
}

// the complex passes along the axes before h, in place on k (nfields fields);
// each axis's stride counts the later axes of the half-spectrum grid, at
// least the M_h / 2 + 1 >= 2 values of axis h
template <class C>
cudaError_t complex_passes(const DipoleReplica& R, C* k, int nfields, bool inverse, cudaStream_t st, bool pdl) {
  for (int s = 0; s < R.h; ++s) {
    const int a = inverse ? R.h - 1 - s : s;
    const int n = R.M[a];
    if (n == 1) continue;
    int64_t stride = 1, outer = nfields;
    for (int b = a + 1; b < 3; ++b) stride *= kdim(R, b);
    for (int b = 0; b < a; ++b) outer *= kdim(R, b);
    if (std::is_same<C, float2>::value && reg_length(n)) {
      const cudaError_t ce = reg_pass_any<C>(n, k, (int)stride, outer, twiddles<C>(R, a), inverse, st, pdl);
      if (ce != cudaSuccess) return ce;
      continue;
    }
    const int G = (int)std::min<int64_t>(stride, lines_per_cta(n, 2 * fft_elems<C>(), fft_pass_lines<C>()));
    const int64_t chunks = (stride + G - 1) / G;
    const size_t sm = (size_t)(2 * G + 1) * n * sizeof(C);
    const cudaError_t ce =
        launch_fft(fft_pass<C>, (unsigned)(outer * chunks), sm, st, pdl, k, (int)stride, G, fast_div((uint32_t)G),
                   fast_div((uint32_t)chunks), R.plan[a], twiddles<C>(R, a), inverse);
    if (ce != cudaSuccess) return ce;
  }
  return cudaSuccess;
}

// forward transform of nfields real fields read through src into the half
// spectrum k (the real pass takes line pairs)
template <class C, class Src>
cudaError_t forward_transform(const DipoleReplica& R, const Src& src, int nfields, C* k, cudaStream_t st, bool pdl,
                              bool sites = false) {
  const int n = R.M[R.h];
  const int O = (int)(R.Mtot / n), nlines = nfields * O, npairs = (nlines + 1) / 2;
  if constexpr (std::is_same<C, float2>::value) {
    if (reg_length(n)) {
      const float2* tw = twiddles<C>(R, R.h);
      cudaError_t ce = cudaSuccess;
#define JAMS_CALL(N) reg_forward<N, Src>(src, nlines, O, sites, tw, k, st, pdl)
      ce = [&]() -> cudaError_t { JAMS_FFT_REG_SWITCH(n, JAMS_CALL) }();
#undef JAMS_CALL
      return ce == cudaSuccess ? complex_passes<C>(R, k, nfields, false, st, pdl) : ce;
    }
  }
  const int G = lines_per_cta(n, fft_elems<C>(), 256);
  const size_t sm = (size_t)(2 * G + 1) * n * sizeof(C);
  const cudaError_t ce = launch_fft(fft_real_forward<C, Src>, (unsigned)((npairs + G - 1) / G), sm, st, pdl, src,
                                    nlines, fast_div((uint32_t)O), G, R.plan[R.h], twiddles<C>(R, R.h), k);
  return ce == cudaSuccess ? complex_passes<C>(R, k, nfields, false, st, pdl) : ce;
}

// inverse transform of the half spectrum k (overwritten) into sink
template <class C, class Sink>
cudaError_t inverse_transform(const DipoleReplica& R, C* k, int nfields, const Sink& sink, cudaStream_t st, bool pdl,
                              bool sites = false) {
  const cudaError_t ce = complex_passes<C>(R, k, nfields, true, st, pdl);
  if (ce != cudaSuccess) return ce;
  const int n = R.M[R.h];
  const int O = (int)(R.Mtot / n), nlines = nfields * O, npairs = (nlines + 1) / 2;
  if constexpr (std::is_same<C, float2>::value) {
    if (reg_length(n)) {
      const float2* tw = twiddles<C>(R, R.h);
#define JAMS_CALL(N) reg_inverse<N, Sink>(k, nlines, O, sites, tw, sink, st, pdl)
      JAMS_FFT_REG_SWITCH(n, JAMS_CALL)
#undef JAMS_CALL
    }
  }
  const int G = lines_per_cta(n, fft_elems<C>(), 256);
  const size_t sm = (size_t)(2 * G + 1) * n * sizeof(C);
  return launch_fft(fft_real_inverse<C, Sink>, (unsigned)((npairs + G - 1) / G), sm, st, pdl, (const C*)k, nlines,
                    fast_div((uint32_t)O), G, R.plan[R.h], twiddles<C>(R, R.h), sink);
}

// the non-zero tensor entries of basis pair (bi, bj) on replica grid R:
// grid index and (xx, xy, xz, yy, yz, zz) x mu0 / (4 pi a^3) / prod(M)
bool tensor_entries(const DipoleGeometry& g, const int periodic[3], const DipoleReplica& R, int bi, int bj,
                    std::vector<int64_t>& idx, std::vector<double>& vals, std::string& err) {
  // reciprocal vectors of A: |fractional coordinate k| <= |r| |b_k|
  const double* A = g.A;
  const double c[3][3] = {{A[4] * A[8] - A[5] * A[7], A[5] * A[6] - A[3] * A[8], A[3] * A[7] - A[4] * A[6]},
                          {A[7] * A[2] - A[8] * A[1], A[8] * A[0] - A[6] * A[2], A[6] * A[1] - A[7] * A[0]},
                          {A[1] * A[5] - A[2] * A[4], A[2] * A[3] - A[0] * A[5], A[0] * A[4] - A[1] * A[3]}};
  const double vol = A[0] * c[0][0] + A[1] * c[0][1] + A[2] * c[0][2];
  if (!(std::fabs(vol) > 0.0)) {
    err = "dipole: lattice vectors are degenerate";
    return false;
  }
  const double rc = g.r_cutoff + g.tolerance;
  const double w0 = (4.0 * kPiD * 1e-7 / kJoule2meVD) / (4.0 * kPiD * g.a * g.a * g.a) /
                    (double)(R.M[0] * (int64_t)R.M[1] * R.M[2]);
  int lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    const double bk = std::sqrt(c[k][0] * c[k][0] + c[k][1] * c[k][1] + c[k][2] * c[k][2]) / std::fabs(vol);
    const int E = (int)std::ceil(rc * bk) + 1;
    if (periodic[k]) {
      if (2 * E + 1 >= R.L[k]) {
        lo[k] = 0;
        hi[k] = R.L[k] - 1;
      } else {
        lo[k] = -E;
        hi[k] = E;
      }
    } else {
      lo[k] = -std::min(E, R.L[k] - 1);
      hi[k] = std::min(E, R.L[k] - 1);
    }
  }
  const double* fi = g.frac[bi];
  const double* fj = g.frac[bj];
  for (int e0 = lo[0]; e0 <= hi[0]; ++e0)
    for (int e1 = lo[1]; e1 <= hi[1]; ++e1)
      for (int e2 = lo[2]; e2 <= hi[2]; ++e2) {
        const int e[3] = {e0, e1, e2};
        double x[3];
        bool zero = true;
        for (int k = 0; k < 3; ++k) {
          x[k] = e[k] + fi[k] - fj[k];
          if (periodic[k]) {
            x[k] -= R.L[k] * std::floor(x[k] / R.L[k] + 0.5);
            if (((e[k] % R.L[k]) + R.L[k]) % R.L[k] != 0) zero = false;
          } else if (e[k] != 0) {
            zero = false;
          }
        }
        if (zero && bi == bj) continue;   // self interaction
        double r[3];
        for (int cc = 0; cc < 3; ++cc) r[cc] = x[0] * A[cc] + x[1] * A[3 + cc] + x[2] * A[6 + cc];
        const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        if (!(r2 > 0.0)) {
          err = "dipole: two sites at the same position";
          return false;
        }
        if (r2 > rc * rc) continue;
        int64_t n = 0;
        for (int k = 0; k < 3; ++k) {
          const int nk = ((e[k] % R.M[k]) + R.M[k]) % R.M[k];
          n = n * R.M[k] + nk;
        }
        const double r5 = std::pow(std::sqrt(r2), 5);
        idx.push_back(n);
        vals.push_back(w0 * (3.0 * r[0] * r[0] - r2) / r5);
        vals.push_back(w0 * (3.0 * r[0] * r[1]) / r5);
        vals.push_back(w0 * (3.0 * r[0] * r[2]) / r5);
        vals.push_back(w0 * (3.0 * r[1] * r[1] - r2) / r5);
        vals.push_back(w0 * (3.0 * r[1] * r[2]) / r5);
        vals.push_back(w0 * (3.0 * r[2] * r[2] - r2) / r5);
      }
  return true;
}

std::string cuda_msg(cudaError_t e, const char* what) { return std::string(what) + ": " + cudaGetErrorString(e); }

}  // namespace

DipoleField* dipole_create(const DipoleGeometry& g, int nb, const int periodic[3], const double* mus,
                           const std::vector<DipoleReplicaSpec>& reps, bool fp64, std::string& err) {
  if (nb < 1 || nb > kMaxBasis) {
    err = "dipole: bad basis size";
    return nullptr;
  }
  if (!(g.a > 0.0) || !(g.r_cutoff > 0.0) || !(g.tolerance >= 0.0)) {
    err = "dipole: lattice_parameter and r_cutoff must be positive";
    return nullptr;
  }
  cudaGetLastError();   // errors below are this call's own
  DipoleField* D = new DipoleField();
  D->fp64 = fp64;
  D->nb = nb;
  for (int b = 0; b < nb; ++b) D->mus.v[b] = mus[b];
  const size_t real = fp64 ? sizeof(double) : sizeof(float);
  const size_t cplx = 2 * real;
  for (const DipoleReplicaSpec& spec : reps) {
    DipoleReplica* R = new DipoleReplica();
    D->reps.push_back(R);
    R->offset = spec.offset;
    for (int k = 0; k < 3; ++k) {
      R->L[k] = spec.L[k];
      R->M[k] = periodic[k] ? spec.L[k] : (spec.L[k] == 1 ? 1 : 2 * spec.L[k]);
    }
    const double rmax = dipole_max_radius(g.A, R->L, periodic);
    if (g.r_cutoff > rmax) {
      err = "dipole: r_cutoff " + std::to_string(g.r_cutoff) +
            " is larger than the inradius of the periodic supercell (" + std::to_string(rmax) + ")";
      delete D;
      return nullptr;
    }
    R->Mtot = (int64_t)R->M[0] * R->M[1] * R->M[2];
    R->h = 0;
    for (int k = 0; k < 3; ++k)
      if (R->M[k] > 1) R->h = k;
    R->Mq = R->Mtot / R->M[R->h] * (R->M[R->h] / 2 + 1);
    if ((int64_t)std::max(3 * nb, 6) * R->Mtot >= ((int64_t)1 << 31)) {
      err = "dipole: the FFT grid of " + std::to_string(R->Mtot) + " cells is too large (fields x cells >= 2^31)";
      delete D;
      return nullptr;
    }
    cudaError_t ce = cudaSuccess;
    for (int k = 0; k < 3 && ce == cudaSuccess; ++k) {
      const int n = R->M[k];
      // one line of a shared-memory pass, two buffers and the twiddle table,
      // within a CTA's 227 KB: 4842 points in FP64, the precision of the
      // tensors' transforms in either form
      const int max_axis = (int)(227 * 1024 / (3 * sizeof(double2)));
      if (n > max_axis) {
        err = "dipole: a grid axis of " + std::to_string(n) + " cells is longer than the transform supports (" +
              std::to_string(max_axis) + ")";
        delete D;
        return nullptr;
      }
      R->plan[k] = fft_plan(n);
      std::vector<double2> td(n);
      std::vector<float2> tf(n);
      for (int t = 0; t < n; ++t) {
        const double ang = 2.0 * kPiD * (double)t / (double)n;
        td[t] = make_double2(std::cos(ang), -std::sin(ang));
        tf[t] = make_float2((float)td[t].x, (float)td[t].y);
      }
      ce = R->twd[k].alloc(n);
      if (ce == cudaSuccess) ce = R->twf[k].alloc(n);
      if (ce == cudaSuccess) ce = cudaMemcpy(R->twd[k].p, td.data(), n * sizeof(double2), cudaMemcpyHostToDevice);
      if (ce == cudaSuccess) ce = cudaMemcpy(R->twf[k].p, tf.data(), n * sizeof(float2), cudaMemcpyHostToDevice);
    }
    if (ce == cudaSuccess) ce = R->ks.alloc((size_t)3 * nb * R->Mq * cplx);
    if (ce == cudaSuccess) ce = R->kh.alloc((size_t)3 * nb * R->Mq * cplx);
    if (ce == cudaSuccess) ce = R->wd.alloc((size_t)nb * 6 * R->Mq * real);
    if (ce == cudaSuccess) ce = R->wo.alloc((size_t)std::max(nb * (nb - 1) / 2, 1) * 6 * R->Mq * cplx);
    if (ce != cudaSuccess) {
      err = cuda_msg(ce, "dipole: allocating grids");
      delete D;
      return nullptr;
    }
    // tensors: scatter the in-cutoff entries onto a zero grid, transform
    // (double), keep in the replica's precision
    Dev<double> tgrid;
    Dev<double2> tk;
    Dev<int64_t> didx;
    Dev<double> dval;
    ce = tgrid.alloc((size_t)6 * R->Mtot);
    if (ce == cudaSuccess) ce = tk.alloc((size_t)6 * R->Mq);
    int pair = 0;
    for (int bi = 0; bi < nb && ce == cudaSuccess && err.empty(); ++bi)
      for (int bj = bi; bj < nb && ce == cudaSuccess && err.empty(); ++bj) {
        std::vector<int64_t> idx;
        std::vector<double> vals;
        if (!tensor_entries(g, periodic, *R, bi, bj, idx, vals, err)) break;
        ce = cudaMemset(tgrid.p, 0, tgrid.n * sizeof(double));
        if (ce == cudaSuccess && !idx.empty()) {
          ce = didx.alloc(idx.size());
          if (ce == cudaSuccess) ce = dval.alloc(vals.size());
          if (ce == cudaSuccess) ce = cudaMemcpy(didx.p, idx.data(), idx.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
          if (ce == cudaSuccess) ce = cudaMemcpy(dval.p, vals.data(), vals.size() * sizeof(double), cudaMemcpyHostToDevice);
          if (ce == cudaSuccess) {
            dip_tensor_scatter<<<blocks((int64_t)idx.size()), kDipBlock>>>(didx.p, dval.p, (int64_t)idx.size(),
                                                                           R->Mtot, tgrid.p);
            ce = cudaGetLastError();
          }
        }
        if (ce != cudaSuccess) break;
        ce = forward_transform<double2>(*R, GridSource{tgrid.p, R->Mtot, R->M[R->h]}, 6, tk.p, 0, false);
        if (ce != cudaSuccess) break;
        const int64_t n = 6 * R->Mq;
        unsigned char* rdst = bi == bj ? R->wd.p + (size_t)bi * 6 * R->Mq * real : nullptr;
        unsigned char* cdst = bi == bj ? nullptr : R->wo.p + (size_t)(pair++) * 6 * R->Mq * cplx;
        if (fp64)
          dip_store_tensor<double2, double><<<blocks(n), kDipBlock>>>(
              tk.p, reinterpret_cast<double*>(rdst), reinterpret_cast<double2*>(cdst), n);
        else
          dip_store_tensor<float2, float><<<blocks(n), kDipBlock>>>(
              tk.p, reinterpret_cast<float*>(rdst), reinterpret_cast<float2*>(cdst), n);
        ce = cudaGetLastError();
      }
    if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    if (ce != cudaSuccess && err.empty()) err = cuda_msg(ce, "dipole: building tensors");
    if (!err.empty()) {
      delete D;
      return nullptr;
    }
  }
  return D;
}

void dipole_destroy(DipoleField* d) { delete d; }

int64_t dipole_launches(const DipoleField* d) {
  int64_t n = 0;
  for (const auto* R : d->reps) {
    int passes = 0;
    for (int a = 0; a < R->h; ++a) passes += R->M[a] > 1;
    n += 3 + 2 * passes;
  }
  return n;
}

size_t dipole_device_bytes(const DipoleField* d) {
  size_t b = 0;
  for (const auto* R : d->reps) b += R->ks.n + R->kh.n + R->wd.n + R->wo.n;
  return b;
}

namespace {

GridCells grid_cells(const DipoleReplica& R, int nb, int64_t npad) {
  GridCells gc;
  for (int k = 0; k < 3; ++k) {
    gc.L[k] = R.L[k];
    gc.M[k] = R.M[k];
  }
  gc.dM1 = fast_div((uint32_t)R.M[1]);
  gc.dM2 = fast_div((uint32_t)R.M[2]);
  gc.dnb = fast_div((uint32_t)nb);
  gc.nb = nb;
  gc.h = R.h;
  gc.npad = npad;
  gc.offset = R.offset;
  return gc;
}

template <class Real, class C>
std::string compute_replica(const DipoleField* D, DipoleReplica* R, const void* s, void* h, int64_t npad,
                            cudaStream_t st) {
  const int nb = D->nb;
  C* ks = reinterpret_cast<C*>(R->ks.p);
  C* kh = reinterpret_cast<C*>(R->kh.p);
  const GridCells gc = grid_cells(*R, nb, npad);
  const SpinSource<Real> src{static_cast<const Real*>(s), gc, R->M[R->h]};
  // basis-site pairs for the real passes: an even basis and even plane
  // offsets (8-byte aligned pairs)
  const bool sites = nb % 2 == 0 && npad % 2 == 0 && R->offset % 2 == 0;
  cudaError_t ce = forward_transform<C>(*R, src, 3 * nb, ks, st, true, sites);
  if (ce != cudaSuccess) return cuda_msg(ce, "dipole: forward transform");
  ce = launch_convolve<C, Real>(nb, ks, reinterpret_cast<const Real*>(R->wd.p), reinterpret_cast<const C*>(R->wo.p),
                                kh, R->Mq, D->mus, st);
  if (ce != cudaSuccess) return cuda_msg(ce, "dipole: k-space product");
  const FieldSink<Real> sink{static_cast<Real*>(h), gc, R->M[R->h], D->mus};
  ce = inverse_transform<C>(*R, kh, 3 * nb, sink, st, true, sites);
  if (ce != cudaSuccess) return cuda_msg(ce, "dipole: inverse transform");
  return std::string();
}

}  // namespace

std::string dipole_compute(DipoleField* D, const void* s, void* h, int64_t npad, cudaStream_t st) {
  for (DipoleReplica* R : D->reps) {
    const std::string e = D->fp64 ? compute_replica<double, double2>(D, R, s, h, npad, st)
                                  : compute_replica<float, float2>(D, R, s, h, npad, st);
    if (!e.empty()) return e;
  }
  return std::string();
}

}  // namespace jams_llg
