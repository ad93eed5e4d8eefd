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
// normalised by the grid size as there.  cuFFT does the transforms; the
// scatter, the k-space product and the gather are this file's kernels.
// FP32C evaluates in single precision (R2C / C2R, float tensors computed in
// double); FP64 in double.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "llg_dipole.h"

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

const char* cufft_name(cufftResult r) {
  switch (r) {
    case CUFFT_SUCCESS: return "success";
    case CUFFT_INVALID_PLAN: return "invalid plan";
    case CUFFT_ALLOC_FAILED: return "allocation failed";
    case CUFFT_INVALID_VALUE: return "invalid value";
    case CUFFT_INTERNAL_ERROR: return "internal error";
    case CUFFT_EXEC_FAILED: return "execution failed";
    case CUFFT_SETUP_FAILED: return "setup failed";
    case CUFFT_INVALID_SIZE: return "invalid size";
    default: return "cuFFT error";
  }
}

// ------------------------------------------------------------------ kernels

// spins of one replica onto its FFT grid: component c of basis site b at
// grid row (c nb + b); cells outside the lattice (padding) are zero
template <class Real>
__global__ void __launch_bounds__(kDipBlock) dip_scatter(const Real* __restrict__ s, int64_t npad, int64_t offset,
                                                         int L0, int L1, int L2, int nb, int M1, int M2,
                                                         int64_t Mtot, Real* __restrict__ grid) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= Mtot) return;
  const int z = (int)(n % M2);
  const int64_t t = n / M2;
  const int y = (int)(t % M1);
  const int x = (int)(t / M1);
  const bool in = x < L0 && y < L1 && z < L2;
  const int64_t i0 = in ? (((int64_t)x * L1 + y) * L2 + z) * nb : 0;
  for (int b = 0; b < nb; ++b)
    for (int c = 0; c < 3; ++c)
      grid[(int64_t)(c * nb + b) * Mtot + n] = in ? s[c * npad + offset + i0 + b] : Real(0);
}

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

// grid -> SoA field planes of the replica, times mu_i; one thread per
// lattice cell (coalesced reads of every grid row; the basis sites of a cell
// are adjacent in the planes)
template <class Real>
__global__ void __launch_bounds__(kDipBlock) dip_gather(const Real* __restrict__ grid, int64_t Mtot, int L1, int L2,
                                                        int nb, int M1, int M2, int64_t ncells, int64_t offset,
                                                        int64_t npad, MusArr mus, Real* __restrict__ h) {
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncells) return;
  const int z = (int)(cell % L2);
  const int y = (int)((cell / L2) % L1);
  const int x = (int)(cell / ((int64_t)L1 * L2));
  const int64_t n = ((int64_t)x * M1 + y) * M2 + z;
  for (int b = 0; b < nb; ++b) {
    const Real mu = (Real)mus.v[b];
    for (int c = 0; c < 3; ++c)
      h[c * npad + offset + cell * nb + b] = mu * grid[(int64_t)(c * nb + b) * Mtot + n];
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

// A batched 3-D real transform over M with the size-1 axes left out
cufftResult make_plan(cufftHandle* plan, const int M[3], cufftType type, int batch, int64_t* Mq) {
  int dims[3], r = 0;
  for (int k = 0; k < 3; ++k)
    if (M[k] > 1) dims[r++] = M[k];
  if (r == 0) dims[r++] = 1;
  int64_t q = 1;
  for (int k = 0; k < r - 1; ++k) q *= dims[k];
  *Mq = q * (dims[r - 1] / 2 + 1);
  return cufftPlanMany(plan, r, dims, nullptr, 1, 0, nullptr, 1, 0, type, batch);
}

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
  cufftHandle fwd = 0, inv = 0;
  bool have_fwd = false, have_inv = false;
  Dev<unsigned char> grid, ks, kh, wd, wo;   // wd: diagonal tensors (real), wo: i < j (complex)
  size_t work = 0;
  ~DipoleReplica() {
    if (have_fwd) cufftDestroy(fwd);
    if (have_inv) cufftDestroy(inv);
  }
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
    cufftResult fr = make_plan(&R->fwd, R->M, fp64 ? CUFFT_D2Z : CUFFT_R2C, 3 * nb, &R->Mq);
    R->have_fwd = fr == CUFFT_SUCCESS;
    if (fr == CUFFT_SUCCESS) {
      int64_t mq = 0;
      fr = make_plan(&R->inv, R->M, fp64 ? CUFFT_Z2D : CUFFT_C2R, 3 * nb, &mq);
      R->have_inv = fr == CUFFT_SUCCESS;
    }
    if (fr != CUFFT_SUCCESS) {
      err = std::string("dipole: cufftPlanMany: ") + cufft_name(fr);
      delete D;
      return nullptr;
    }
    size_t ws = 0;
    cufftGetSize(R->fwd, &ws);
    R->work = ws;
    cufftGetSize(R->inv, &ws);
    R->work += ws;
    cudaError_t ce = R->grid.alloc((size_t)3 * nb * R->Mtot * real);
    if (ce == cudaSuccess) ce = R->ks.alloc((size_t)3 * nb * R->Mq * cplx);
    if (ce == cudaSuccess) ce = R->kh.alloc((size_t)3 * nb * R->Mq * cplx);
    if (ce == cudaSuccess) ce = R->wd.alloc((size_t)nb * 6 * R->Mq * real);
    if (ce == cudaSuccess) ce = R->wo.alloc((size_t)std::max(nb * (nb - 1) / 2, 1) * 6 * R->Mq * cplx);
    if (ce != cudaSuccess) {
      err = cuda_msg(ce, "dipole: allocating grids");
      delete D;
      return nullptr;
    }
    // tensors: scatter the in-cutoff entries onto a zero grid, D2Z, keep
    cufftHandle tplan;
    int64_t mq6 = 0;
    fr = make_plan(&tplan, R->M, CUFFT_D2Z, 6, &mq6);
    if (fr != CUFFT_SUCCESS) {
      err = std::string("dipole: tensor plan: ") + cufft_name(fr);
      delete D;
      return nullptr;
    }
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
        fr = cufftExecD2Z(tplan, tgrid.p, reinterpret_cast<cufftDoubleComplex*>(tk.p));
        if (fr != CUFFT_SUCCESS) {
          err = std::string("dipole: tensor transform: ") + cufft_name(fr);
          break;
        }
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
    cufftDestroy(tplan);
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
  for (const auto* R : d->reps) b += R->grid.n + R->ks.n + R->kh.n + R->wd.n + R->wo.n + R->work;
  return b;
}

std::string dipole_compute(DipoleField* D, const void* s, void* h, int64_t npad, cudaStream_t st) {
  const int nb = D->nb;
  for (DipoleReplica* R : D->reps) {
    const int64_t ncells = (int64_t)R->L[0] * R->L[1] * R->L[2];
    cufftResult fr = cufftSetStream(R->fwd, st);
    if (fr == CUFFT_SUCCESS) fr = cufftSetStream(R->inv, st);
    if (fr != CUFFT_SUCCESS) return std::string("dipole: cufftSetStream: ") + cufft_name(fr);
    if (D->fp64) {
      double* grid = reinterpret_cast<double*>(R->grid.p);
      auto* ks = reinterpret_cast<cufftDoubleComplex*>(R->ks.p);
      auto* kh = reinterpret_cast<cufftDoubleComplex*>(R->kh.p);
      dip_scatter<double><<<blocks(R->Mtot), kDipBlock, 0, st>>>(static_cast<const double*>(s), npad, R->offset,
                                                                R->L[0], R->L[1], R->L[2], nb, R->M[1], R->M[2],
                                                                R->Mtot, grid);
      fr = cufftExecD2Z(R->fwd, grid, ks);
      if (fr != CUFFT_SUCCESS) return std::string("dipole: D2Z: ") + cufft_name(fr);
      launch_convolve<double2, double>(nb, ks, reinterpret_cast<const double*>(R->wd.p),
                                       reinterpret_cast<const double2*>(R->wo.p), kh, R->Mq, D->mus, st);
      fr = cufftExecZ2D(R->inv, kh, grid);
      if (fr != CUFFT_SUCCESS) return std::string("dipole: Z2D: ") + cufft_name(fr);
      dip_gather<double><<<blocks(ncells), kDipBlock, 0, st>>>(grid, R->Mtot, R->L[1], R->L[2], nb, R->M[1],
                                                               R->M[2], ncells, R->offset, npad, D->mus,
                                                               static_cast<double*>(h));
    } else {
      float* grid = reinterpret_cast<float*>(R->grid.p);
      auto* ks = reinterpret_cast<cufftComplex*>(R->ks.p);
      auto* kh = reinterpret_cast<cufftComplex*>(R->kh.p);
      dip_scatter<float><<<blocks(R->Mtot), kDipBlock, 0, st>>>(static_cast<const float*>(s), npad, R->offset,
                                                               R->L[0], R->L[1], R->L[2], nb, R->M[1], R->M[2],
                                                               R->Mtot, grid);
      fr = cufftExecR2C(R->fwd, grid, ks);
      if (fr != CUFFT_SUCCESS) return std::string("dipole: R2C: ") + cufft_name(fr);
      launch_convolve<float2, float>(nb, ks, reinterpret_cast<const float*>(R->wd.p),
                                     reinterpret_cast<const float2*>(R->wo.p), kh, R->Mq, D->mus, st);
      fr = cufftExecC2R(R->inv, kh, grid);
      if (fr != CUFFT_SUCCESS) return std::string("dipole: C2R: ") + cufft_name(fr);
      dip_gather<float><<<blocks(ncells), kDipBlock, 0, st>>>(grid, R->Mtot, R->L[1], R->L[2], nb, R->M[1],
                                                              R->M[2], ncells, R->offset, npad, D->mus,
                                                              static_cast<float*>(h));
    }
    const cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) return cuda_msg(ce, "dipole kernels");
  }
  return std::string();
}

}  // namespace jams_llg
