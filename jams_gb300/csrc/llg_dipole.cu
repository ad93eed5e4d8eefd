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
#include <vector>

#include "llg_dipole.h"
#include "llg_fft.cuh"

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

// position (x, y, z) of point p of line o along the real axis h (the axes
// after h have one cell)
__device__ __forceinline__ void line_cell(int64_t o, int p, int h, const int M[3], int c[3]) {
  c[0] = c[1] = c[2] = 0;
  c[h] = p;
  for (int a = h - 1; a >= 0; --a) {
    c[a] = (int)(o % M[a]);
    o /= M[a];
  }
}

// the spins of one replica on its FFT grid, read by the forward real pass
// (the scatter fused into it): field f = component * nb + basis site; cells
// outside the lattice (padding) are zero
template <class Real>
struct SpinSource {
  const Real* s;
  int64_t npad, offset;
  int L[3], M[3], h, nb;
  __device__ Real operator()(int64_t f, int64_t o, int p) const {
    int c[3];
    line_cell(o, p, h, M, c);
    if (c[0] >= L[0] || c[1] >= L[1] || c[2] >= L[2]) return Real(0);
    const int m = (int)(f / nb), b = (int)(f % nb);
    return s[m * npad + offset + (((int64_t)c[0] * L[1] + c[1]) * L[2] + c[2]) * nb + b];
  }
};

// a real grid of fields (the tensors at set-up)
struct GridSource {
  const double* g;
  int64_t Mtot;
  int Mh;
  __device__ double operator()(int64_t f, int64_t o, int p) const { return g[f * Mtot + o * Mh + p]; }
};

// the field planes of one replica, written by the inverse real pass (the
// gather fused into it): mu_s times the transform, lattice cells only
template <class Real>
struct FieldSink {
  Real* hp;
  int64_t npad, offset;
  int L[3], M[3], h, nb;
  MusArr mus;
  __device__ void operator()(int64_t f, int64_t o, int p, Real v) const {
    int c[3];
    line_cell(o, p, h, M, c);
    if (c[0] >= L[0] || c[1] >= L[1] || c[2] >= L[2]) return;
    const int m = (int)(f / nb), b = (int)(f % nb);
    hp[m * npad + offset + (((int64_t)c[0] * L[1] + c[1]) * L[2] + c[2]) * nb + b] = (Real)mus.v[b] * v;
  }
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
void launch_convolve(int nb, const C* ks, const Real* wd, const C* wo, C* kh, int64_t Mq, const MusArr& mus,
                     cudaStream_t st) {
  const unsigned g = (unsigned)((Mq + kDipBlock - 1) / kDipBlock);
  switch (nb) {
    case 1: dip_convolve<C, Real, 1><<<g, kDipBlock, 0, st>>>(ks, wd, wo, kh, Mq, mus); break;
    case 2: dip_convolve<C, Real, 2><<<g, kDipBlock, 0, st>>>(ks, wd, wo, kh, Mq, mus); break;
    case 3: dip_convolve<C, Real, 3><<<g, kDipBlock, 0, st>>>(ks, wd, wo, kh, Mq, mus); break;
    default: dip_convolve<C, Real, 4><<<g, kDipBlock, 0, st>>>(ks, wd, wo, kh, Mq, mus); break;
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

// complex values per shared-memory buffer of a transform pass
template <class C>
constexpr int fft_elems() {
  return sizeof(C) == sizeof(float2) ? 4096 : 2048;
}

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

// the complex passes along the axes before h, in place on k (nfields fields)
template <class C>
cudaError_t complex_passes(const DipoleReplica& R, C* k, int nfields, bool inverse, cudaStream_t st) {
  for (int s = 0; s < R.h; ++s) {
    const int a = inverse ? R.h - 1 - s : s;
    const int n = R.M[a];
    if (n == 1) continue;
    int64_t stride = 1, outer = nfields;
    for (int b = a + 1; b < 3; ++b) stride *= kdim(R, b);
    for (int b = 0; b < a; ++b) outer *= kdim(R, b);
    const int G = (int)std::min<int64_t>(stride, fft_batch(n, fft_elems<C>()));
    const size_t sm = (size_t)2 * G * n * sizeof(C);
    cudaError_t ce = allow_smem((const void*)fft_pass<C>, sm);
    if (ce != cudaSuccess) return ce;
    const int64_t grid = outer * ((stride + G - 1) / G);
    fft_pass<C><<<(unsigned)grid, kFftThreads, sm, st>>>(k, outer, (int)stride, G, R.plan[a], twiddles<C>(R, a),
                                                         inverse);
  }
  return cudaGetLastError();
}

// forward transform of nfields real fields read through src into the half
// spectrum k
template <class C, class Src>
cudaError_t forward_transform(const DipoleReplica& R, Src src, int nfields, C* k, cudaStream_t st) {
  const int n = R.M[R.h];
  const int64_t O = R.Mtot / n, nlines = (int64_t)nfields * O;
  const int G = fft_batch(n, fft_elems<C>());
  const size_t sm = (size_t)2 * G * n * sizeof(C);
  cudaError_t ce = allow_smem((const void*)fft_real_forward<C, Src>, sm);
  if (ce != cudaSuccess) return ce;
  fft_real_forward<C, Src><<<(unsigned)((nlines + G - 1) / G), kFftThreads, sm, st>>>(src, nlines, O, G, R.plan[R.h],
                                                                                      twiddles<C>(R, R.h), k);
  ce = cudaGetLastError();
  return ce == cudaSuccess ? complex_passes<C>(R, k, nfields, false, st) : ce;
}

// inverse transform of the half spectrum k (overwritten) into sink
template <class C, class Sink>
cudaError_t inverse_transform(const DipoleReplica& R, C* k, int nfields, Sink sink, cudaStream_t st) {
  cudaError_t ce = complex_passes<C>(R, k, nfields, true, st);
  if (ce != cudaSuccess) return ce;
  const int n = R.M[R.h];
  const int64_t O = R.Mtot / n, nlines = (int64_t)nfields * O;
  const int G = fft_batch(n, fft_elems<C>());
  const size_t sm = (size_t)2 * G * n * sizeof(C);
  ce = allow_smem((const void*)fft_real_inverse<C, Sink>, sm);
  if (ce != cudaSuccess) return ce;
  fft_real_inverse<C, Sink><<<(unsigned)((nlines + G - 1) / G), kFftThreads, sm, st>>>(k, nlines, O, G, R.plan[R.h],
                                                                                       twiddles<C>(R, R.h), sink);
  return cudaGetLastError();
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
    cudaError_t ce = cudaSuccess;
    for (int k = 0; k < 3 && ce == cudaSuccess; ++k) {
      const int n = R->M[k];
      if (n > 7168) {
        err = "dipole: a grid axis of " + std::to_string(n) + " cells is longer than the transform supports (7168)";
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
        ce = forward_transform<double2>(*R, GridSource{tgrid.p, R->Mtot, R->M[R->h]}, 6, tk.p, 0);
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

size_t dipole_device_bytes(const DipoleField* d) {
  size_t b = 0;
  for (const auto* R : d->reps) b += R->ks.n + R->kh.n + R->wd.n + R->wo.n;
  return b;
}

namespace {

template <class Real, class C>
std::string compute_replica(const DipoleField* D, DipoleReplica* R, const void* s, void* h, int64_t npad,
                            cudaStream_t st) {
  const int nb = D->nb;
  C* ks = reinterpret_cast<C*>(R->ks.p);
  C* kh = reinterpret_cast<C*>(R->kh.p);
  SpinSource<Real> src{static_cast<const Real*>(s), npad, R->offset, {R->L[0], R->L[1], R->L[2]},
                       {R->M[0], R->M[1], R->M[2]}, R->h, nb};
  cudaError_t ce = forward_transform<C>(*R, src, 3 * nb, ks, st);
  if (ce != cudaSuccess) return cuda_msg(ce, "dipole: forward transform");
  launch_convolve<C, Real>(nb, ks, reinterpret_cast<const Real*>(R->wd.p), reinterpret_cast<const C*>(R->wo.p), kh,
                           R->Mq, D->mus, st);
  FieldSink<Real> sink{static_cast<Real*>(h), npad, R->offset, {R->L[0], R->L[1], R->L[2]},
                       {R->M[0], R->M[1], R->M[2]}, R->h, nb, D->mus};
  ce = inverse_transform<C>(*R, kh, 3 * nb, sink, st);
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
