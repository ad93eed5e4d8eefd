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
//   scatter the spins onto the grid -> R2C -> h_i(q) = sum_j mu_j G_ij(q) S_j(q)
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

template <class C>
__device__ __forceinline__ C cmad(C acc, C a, C b) {
  acc.x += a.x * b.x - a.y * b.y;
  acc.y += a.x * b.y + a.y * b.x;
  return acc;
}

// h_i(q) = sum_j mu_j G_ij(q) S_j(q) for every k-space point q; G holds the
// six independent components xx, xy, xz, yy, yz, zz
template <class C>
__global__ void __launch_bounds__(kDipBlock) dip_convolve(const C* __restrict__ ks, const C* __restrict__ w,
                                                          C* __restrict__ kh, int nb, int64_t Mq, MusArr mus) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= Mq) return;
  for (int i = 0; i < nb; ++i) {
    C h[3];
    for (int m = 0; m < 3; ++m) h[m].x = h[m].y = 0;
    for (int j = 0; j < nb; ++j) {
      C sj[3];
      for (int m = 0; m < 3; ++m) {
        sj[m] = ks[(int64_t)(m * nb + j) * Mq + q];
        sj[m].x *= mus.v[j];
        sj[m].y *= mus.v[j];
      }
      const C* g = w + (int64_t)((i * nb + j) * 6) * Mq + q;
      const C gxx = g[0], gxy = g[Mq], gxz = g[2 * Mq], gyy = g[3 * Mq], gyz = g[4 * Mq], gzz = g[5 * Mq];
      h[0] = cmad(cmad(cmad(h[0], gxx, sj[0]), gxy, sj[1]), gxz, sj[2]);
      h[1] = cmad(cmad(cmad(h[1], gxy, sj[0]), gyy, sj[1]), gyz, sj[2]);
      h[2] = cmad(cmad(cmad(h[2], gxz, sj[0]), gyz, sj[1]), gzz, sj[2]);
    }
    for (int m = 0; m < 3; ++m) kh[(int64_t)(m * nb + i) * Mq + q] = h[m];
  }
}

// grid -> SoA field planes of the replica, times mu_i
template <class Real>
__global__ void __launch_bounds__(kDipBlock) dip_gather(const Real* __restrict__ grid, int64_t Mtot, int L1, int L2,
                                                        int nb, int M1, int M2, int64_t nspins, int64_t offset,
                                                        int64_t npad, MusArr mus, Real* __restrict__ h) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nspins) return;
  const int b = (int)(i % nb);
  const int64_t cell = i / nb;
  const int z = (int)(cell % L2);
  const int y = (int)((cell / L2) % L1);
  const int x = (int)(cell / ((int64_t)L1 * L2));
  const int64_t n = ((int64_t)x * M1 + y) * M2 + z;
  const Real mu = (Real)mus.v[b];
  for (int c = 0; c < 3; ++c) h[c * npad + offset + i] = mu * grid[(int64_t)(c * nb + b) * Mtot + n];
}

__global__ void dip_tensor_scatter(const int64_t* __restrict__ idx, const double* __restrict__ vals, int64_t n,
                                   int64_t Mtot, double* __restrict__ grid) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  for (int c = 0; c < 6; ++c) grid[c * Mtot + idx[e]] = vals[6 * e + c];
}

__global__ void dip_to_float(const double2* __restrict__ a, float2* __restrict__ b, int64_t n) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) b[e] = make_float2((float)a[e].x, (float)a[e].y);
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
  Dev<unsigned char> grid, ks, kh, w;
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
    if (ce == cudaSuccess) ce = R->w.alloc((size_t)nb * nb * 6 * R->Mq * cplx);
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
    for (int bi = 0; bi < nb && ce == cudaSuccess && err.empty(); ++bi)
      for (int bj = 0; bj < nb && ce == cudaSuccess && err.empty(); ++bj) {
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
        unsigned char* dst = R->w.p + (size_t)(bi * nb + bj) * 6 * R->Mq * cplx;
        if (fp64) {
          ce = cudaMemcpy(dst, tk.p, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice);
        } else {
          dip_to_float<<<blocks(n), kDipBlock>>>(tk.p, reinterpret_cast<float2*>(dst), n);
          ce = cudaGetLastError();
        }
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
  for (const auto* R : d->reps) b += R->grid.n + R->ks.n + R->kh.n + R->w.n + R->work;
  return b;
}

std::string dipole_compute(DipoleField* D, const void* s, void* h, int64_t npad, cudaStream_t st) {
  const int nb = D->nb;
  for (DipoleReplica* R : D->reps) {
    const int64_t nspins = (int64_t)R->L[0] * R->L[1] * R->L[2] * nb;
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
      dip_convolve<double2><<<blocks(R->Mq), kDipBlock, 0, st>>>(ks, reinterpret_cast<const double2*>(R->w.p), kh,
                                                                nb, R->Mq, D->mus);
      fr = cufftExecZ2D(R->inv, kh, grid);
      if (fr != CUFFT_SUCCESS) return std::string("dipole: Z2D: ") + cufft_name(fr);
      dip_gather<double><<<blocks(nspins), kDipBlock, 0, st>>>(grid, R->Mtot, R->L[1], R->L[2], nb, R->M[1],
                                                               R->M[2], nspins, R->offset, npad, D->mus,
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
      dip_convolve<float2><<<blocks(R->Mq), kDipBlock, 0, st>>>(ks, reinterpret_cast<const float2*>(R->w.p), kh, nb,
                                                               R->Mq, D->mus);
      fr = cufftExecC2R(R->inv, kh, grid);
      if (fr != CUFFT_SUCCESS) return std::string("dipole: C2R: ") + cufft_name(fr);
      dip_gather<float><<<blocks(nspins), kDipBlock, 0, st>>>(grid, R->Mtot, R->L[1], R->L[2], nb, R->M[1],
                                                              R->M[2], nspins, R->offset, npad, D->mus,
                                                              static_cast<float*>(h));
    }
    const cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) return cuda_msg(ce, "dipole kernels");
  }
  return std::string();
}

}  // namespace jams_llg
