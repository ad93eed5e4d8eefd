// The reference's GPU Heun path, restated for the "ref-GPU" baseline column
// of bench.py.  Measurement infrastructure: libjams_llg.so never links it.
//
// The reference's CUDA sources cannot be compiled where the benchmark runs
// (its sources are not there), so this file restates the algorithm and the
// launch structure of CUDAHeunLLGSolver::run
// (src/jams/solvers/cuda_llg_heun.cu:64-122) in code of its own, calling the
// same libraries:
//   - copy s -> s_old (device to device);
//   - thermostat update: cuRAND normals for the 3N components, scaled by
//     sigma sqrt(T) (src/jams/thermostats/cuda_thermostat_classical.cc:49-56);
//     at T = 0 a memset;
//   - compute_fields (src/jams/cuda/cuda_solver.cc:11-26): each term's field
//     into its own N x 3 buffer - exchange by cuSPARSE CSR SpMV (generic API,
//     CSR_ALG1, int32 indices; src/jams/containers/sparse_matrix.h:343-430),
//     uniaxial, cubic and applied field by one kernel each - then a blocking
//     cudaMemcpy of the first into h and cublasDaxpy of the others;
//   - kernel A: rhs, ds = rhs/2, s = unit(s + dt rhs); compute_fields again;
//     kernel B: ds += rhs/2, s = unit(s_old + dt ds), each with the
//     reference's layout of 84 x 3 threads per block, one thread per spin
//     component of the AoS double arrays, staged in shared memory
//     (src/jams/solvers/cuda_llg_heun_kernel.cuh:8-106).
// The exchange matrix is the reference's 3N x 3N CSR: row 3i+m holds the
// nonzero J_mn of every neighbour j of i at column 3j+n, ascending
// (src/jams/hamiltonian/sparse_interaction.cc:25-34).
//
// Heun, FP64, one replica; exchange, uniaxial, cubic and static applied-field
// terms.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <curand.h>
#include <cusparse.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../include/jams_llg.h"

namespace {

constexpr double kBoltzmannIU = 0.0861733326;   // src/jams/helpers/consts.h:32
thread_local std::string g_err;

struct Term {
  int kind;
  int order;
  double* field = nullptr;        // N x 3 doubles (device)
  double* K = nullptr;            // per spin (device)
  double* axis = nullptr;         // per spin: 3 (uniaxial) or 9 (cubic) (device)
  double B[3] = {0, 0, 0};
  // exchange
  int* row = nullptr;
  int* col = nullptr;
  double* val = nullptr;
  int64_t nnz = 0;
  cusparseSpMatDescr_t A = nullptr;
  cusparseDnVecDescr_t x = nullptr, y = nullptr;
  void* buffer = nullptr;
  size_t buffer_size = 0;
};

struct RefGpu {
  int n = 0;
  double dt = 0.0, temperature = 0.0;
  double *s = nullptr, *s_old = nullptr, *h = nullptr, *ds = nullptr, *noise = nullptr, *sigma = nullptr;
  double *gyro = nullptr, *mus = nullptr, *alpha = nullptr;
  std::vector<Term> terms;
  cudaStream_t stream = nullptr;
  cusparseHandle_t sp = nullptr;
  cublasHandle_t bl = nullptr;
  curandGenerator_t rng = nullptr;

  ~RefGpu() {
    for (auto& t : terms) {
      if (t.A) cusparseDestroySpMat(t.A);
      if (t.x) cusparseDestroyDnVec(t.x);
      if (t.y) cusparseDestroyDnVec(t.y);
      for (void* p : {(void*)t.field, (void*)t.K, (void*)t.axis, (void*)t.row, (void*)t.col, (void*)t.val, t.buffer})
        if (p) cudaFree(p);
    }
    for (double* p : {s, s_old, h, ds, noise, sigma, gyro, mus, alpha})
      if (p) cudaFree(p);
    if (rng) curandDestroyGenerator(rng);
    if (bl) cublasDestroy(bl);
    if (sp) cusparseDestroy(sp);
    if (stream) cudaStreamDestroy(stream);
  }
};

int fail(const std::string& m) {
  g_err = m;
  return -1;
}

template <typename T>
cudaError_t upload(T** dst, const std::vector<T>& v) {
  cudaError_t e = cudaMalloc((void**)dst, std::max<size_t>(v.size(), 1) * sizeof(T));
  if (e == cudaSuccess && !v.empty()) e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

// ------------------------------------------------------------------ kernels

// noise = sigma sqrt(T) noise
__global__ void scale_noise(int n3, const double* sigma, double sqrt_t, double* noise) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n3) noise[k] = sigma[k] * sqrt_t * noise[k];
}

// h = K p (s.a)^(p-1) a  (uniaxial_anisotropy.cc:155-163)
__global__ void uniaxial_field(int n, int power, const double* K, const double* axis, const double* s, double* h) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* a = axis + 3 * i;
  const double d = a[0] * s[3 * i] + a[1] * s[3 * i + 1] + a[2] * s[3 * i + 2];
  const double pre = K[i] * power * pow(d, power - 1);
  for (int m = 0; m < 3; ++m) h[3 * i + m] = pre * a[m];
}

// cubic K1 / K2 field (cubic_anisotropy.cc:197-226)
__global__ void cubic_field(int n, int order, const double* K, const double* axis, const double* s, double* h) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* u = axis + 9 * i;
  const double* v = u + 3;
  const double* w = u + 6;
  const double* sp = s + 3 * i;
  const double Su = u[0] * sp[0] + u[1] * sp[1] + u[2] * sp[2];
  const double Sv = v[0] * sp[0] + v[1] * sp[1] + v[2] * sp[2];
  const double Sw = w[0] * sp[0] + w[1] * sp[1] + w[2] * sp[2];
  const double pre = 2.0 * K[i];
  for (int m = 0; m < 3; ++m) {
    double x;
    if (order == 1)
      x = u[m] * Su * (Sv * Sv + Sw * Sw) + v[m] * Sv * (Sw * Sw + Su * Su) + w[m] * Sw * (Su * Su + Sv * Sv);
    else
      x = u[m] * Su * (Sv * Sv) * (Sw * Sw) + v[m] * Sv * (Sw * Sw) * (Su * Su) + w[m] * Sw * (Su * Su) * (Sv * Sv);
    h[3 * i + m] = pre * x;
  }
}

// h = mu_s B  (applied_field.cc:146-148)
__global__ void applied_field(int n, const double* mus, double Bx, double By, double Bz, double* h) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  h[3 * i] = mus[i] * Bx;
  h[3 * i + 1] = mus[i] * By;
  h[3 * i + 2] = mus[i] * Bz;
}

// one Heun half-step in the reference's layout: blockDim (84, 3), thread
// (x, c) handles component c of spin 84 blockIdx.x + x; the three components
// of s and h' = h / mu_s + noise meet in shared memory.  B: corrector.
template <bool B>
__global__ void heun_half(double* s, double* ds, const double* s_old, const double* h, const double* noise,
                          const double* gyro, const double* mus, const double* alpha, double dt, int n) {
  __shared__ double ss[85 * 3];
  __shared__ double hh[85 * 3];
  const int x = threadIdx.x, c = threadIdx.y;
  const int i = blockIdx.x * blockDim.x + x;
  const bool on = i < n;
  const int p0 = 3 * x + c, p1 = 3 * x + (c + 1) % 3, p2 = 3 * x + (c + 2) % 3;
  const int g = 3 * i + c;
  if (on) {
    hh[p0] = h[g] / mus[i] + noise[g];
    ss[p0] = s[g];
  }
  __syncthreads();
  double v = 0.0;
  if (on) {
    const double rhs = -gyro[i] * ((ss[p1] * hh[p2] - ss[p2] * hh[p1]) +
                                   alpha[i] * (ss[p1] * (ss[p0] * hh[p1] - ss[p1] * hh[p0]) -
                                               ss[p2] * (ss[p2] * hh[p0] - ss[p0] * hh[p2])));
    if (B) {
      ds[g] = ds[g] + 0.5 * rhs;
      v = s_old[g] + dt * ds[g];
    } else {
      ds[g] = 0.5 * rhs;
      v = ss[p0] + dt * rhs;
    }
  }
  __syncthreads();
  if (on) ss[p0] = v;
  __syncthreads();
  if (on) s[g] = ss[p0] * rsqrt(ss[3 * x] * ss[3 * x] + ss[3 * x + 1] * ss[3 * x + 1] + ss[3 * x + 2] * ss[3 * x + 2]);
}

// ------------------------------------------------------------------- host

// 3N x 3N CSR of an exchange template on an L0 x L1 x L2 lattice of nb sites
int build_csr(const llg_desc* d, const llg_term& T, std::vector<int>& row, std::vector<int>& col,
              std::vector<double>& val) {
  const int* L = d->replicas[0].L;
  const int nb = d->nb;
  const int64_t n = (int64_t)L[0] * L[1] * L[2] * nb;
  row.assign(3 * n + 1, 0);
  col.clear();
  val.clear();
  std::vector<std::pair<int64_t, double>> rowbuf[3];
  for (int64_t i = 0; i < n; ++i) {
    const int b = (int)(i % nb);
    int64_t cell = i / nb;
    const int c2 = (int)(cell % L[2]);
    cell /= L[2];
    const int c1 = (int)(cell % L[1]);
    const int c0 = (int)(cell / L[1]);
    for (auto& r : rowbuf) r.clear();
    for (int e = 0; e < T.n_int; ++e) {
      if (T.bi[e] != b) continue;
      int c[3] = {c0 + T.T[3 * e], c1 + T.T[3 * e + 1], c2 + T.T[3 * e + 2]};
      bool ok = true;
      for (int l = 0; l < 3; ++l) {
        if (d->periodic[l]) c[l] = ((c[l] % L[l]) + L[l]) % L[l];
        else if (c[l] < 0 || c[l] >= L[l]) ok = false;
      }
      if (!ok) continue;
      const int64_t j = (((int64_t)c[0] * L[1] + c[1]) * L[2] + c[2]) * nb + T.bj[e];
      for (int m = 0; m < 3; ++m)
        for (int q = 0; q < 3; ++q) {
          const double v = T.J[9 * e + 3 * m + q];
          if (v != 0.0) rowbuf[m].push_back({3 * j + q, v});
        }
    }
    for (int m = 0; m < 3; ++m) {
      auto& r = rowbuf[m];
      std::sort(r.begin(), r.end(), [](const auto& a, const auto& b2) { return a.first < b2.first; });
      for (size_t k = 0; k < r.size(); ++k) {
        if (k > 0 && r[k].first == r[k - 1].first) {
          val.back() += r[k].second;
          continue;
        }
        col.push_back((int)r[k].first);
        val.push_back(r[k].second);
      }
      if (col.size() > (size_t)INT32_MAX) return fail("the exchange matrix exceeds the reference's int32 CSR");
      row[3 * i + m + 1] = (int)col.size();
    }
  }
  return 0;
}

void launch_term_field(RefGpu* g, Term& t) {
  const int nb = (g->n + 63) / 64;
  switch (t.kind) {
    case LLG_TERM_EXCHANGE: {
      const double one = 1.0, zero = 0.0;
      cusparseSetStream(g->sp, g->stream);
      cusparseDnVecSetValues(t.x, g->s);
      cusparseDnVecSetValues(t.y, t.field);
      size_t need = 0;
      cusparseSpMV_bufferSize(g->sp, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, t.A, t.x, &zero, t.y, CUDA_R_64F,
                              CUSPARSE_SPMV_CSR_ALG1, &need);
      if (need > t.buffer_size) {
        if (t.buffer) cudaFree(t.buffer);
        cudaMalloc(&t.buffer, need);
        t.buffer_size = need;
      }
      cusparseSpMV(g->sp, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, t.A, t.x, &zero, t.y, CUDA_R_64F,
                   CUSPARSE_SPMV_CSR_ALG1, t.buffer);
      break;
    }
    case LLG_TERM_UNIAXIAL:
      uniaxial_field<<<nb, 64, 0, g->stream>>>(g->n, t.order, t.K, t.axis, g->s, t.field);
      break;
    case LLG_TERM_CUBIC:
      cubic_field<<<nb, 64, 0, g->stream>>>(g->n, t.order, t.K, t.axis, g->s, t.field);
      break;
    default:
      applied_field<<<nb, 64, 0, g->stream>>>(g->n, g->mus, t.B[0], t.B[1], t.B[2], t.field);
      break;
  }
}

// h = field of term 0 (blocking copy) + daxpy of the others
void compute_fields(RefGpu* g) {
  for (auto& t : g->terms) launch_term_field(g, t);
  cudaMemcpy(g->h, g->terms[0].field, (size_t)g->n * 3 * sizeof(double), cudaMemcpyDeviceToDevice);
  const double one = 1.0;
  cublasSetStream(g->bl, g->stream);
  for (size_t k = 1; k < g->terms.size(); ++k) cublasDaxpy(g->bl, 3 * g->n, &one, g->terms[k].field, 1, g->h, 1);
}

void step(RefGpu* g) {
  const size_t bytes = (size_t)g->n * 3 * sizeof(double);
  cudaMemcpyAsync(g->s_old, g->s, bytes, cudaMemcpyDeviceToDevice, g->stream);
  if (g->temperature == 0.0) {
    cudaMemset(g->noise, 0, bytes);
  } else {
    const size_t n3 = (size_t)g->n * 3;
    curandSetStream(g->rng, g->stream);
    curandGenerateNormalDouble(g->rng, g->noise, n3 + (n3 % 2), 0.0, 1.0);
    scale_noise<<<(unsigned)((n3 + 255) / 256), 256, 0, g->stream>>>((int)n3, g->sigma, std::sqrt(g->temperature),
                                                                       g->noise);
  }
  const dim3 block(84, 3);
  const dim3 grid((unsigned)((g->n + 83) / 84));
  compute_fields(g);
  heun_half<false><<<grid, block, 0, g->stream>>>(g->s, g->ds, g->s_old, g->h, g->noise, g->gyro, g->mus, g->alpha,
                                                 g->dt, g->n);
  compute_fields(g);
  heun_half<true><<<grid, block, 0, g->stream>>>(g->s, g->ds, g->s_old, g->h, g->noise, g->gyro, g->mus, g->alpha,
                                                g->dt, g->n);
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) const char* refgpu_last_error() { return g_err.c_str(); }

__attribute__((visibility("default"))) int refgpu_create(const llg_desc* d, void** out) {
  if (!d || !out || d->n_replicas < 1 || !d->replicas) return fail("bad descriptor");
  if (d->integrator != LLG_HEUN) return fail("the reference GPU path here is Heun");
  RefGpu* g = new RefGpu();
  const llg_replica& R = d->replicas[0];
  g->n = R.L[0] * R.L[1] * R.L[2] * d->nb;
  g->dt = d->dt;
  g->temperature = R.temperature;
  const int n = g->n, nb = d->nb;
  std::vector<double> mus(n), gyro(n), alpha(n), sigma(3 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    const int b = i % nb;
    mus[i] = d->mus[b];
    gyro[i] = d->gyro[b];
    alpha[i] = d->alpha[b];
    const double den = d->gilbert_prefactor ? 1.0 + alpha[i] * alpha[i] : 1.0;
    const double sg = std::sqrt((2.0 * kBoltzmannIU * alpha[i]) / (mus[i] * gyro[i] * d->dt * den));
    for (int m = 0; m < 3; ++m) sigma[3 * (size_t)i + m] = sg;
  }
  cudaError_t ce = cudaSuccess;
  const size_t bytes = (size_t)n * 3 * sizeof(double);
  for (double** p : {&g->s, &g->s_old, &g->h, &g->ds, &g->noise})
    if (ce == cudaSuccess) ce = cudaMalloc((void**)p, bytes + 16);
  if (ce == cudaSuccess) ce = upload(&g->sigma, sigma);
  if (ce == cudaSuccess) ce = upload(&g->mus, mus);
  if (ce == cudaSuccess) ce = upload(&g->gyro, gyro);
  if (ce == cudaSuccess) ce = upload(&g->alpha, alpha);
  if (ce == cudaSuccess) ce = cudaStreamCreate(&g->stream);
  if (ce != cudaSuccess) {
    delete g;
    return fail(std::string("CUDA: ") + cudaGetErrorString(ce));
  }
  if (cusparseCreate(&g->sp) != CUSPARSE_STATUS_SUCCESS || cublasCreate(&g->bl) != CUBLAS_STATUS_SUCCESS ||
      curandCreateGenerator(&g->rng, CURAND_RNG_PSEUDO_XORWOW) != CURAND_STATUS_SUCCESS) {
    delete g;
    return fail("library handle creation failed");
  }
  curandSetPseudoRandomGeneratorSeed(g->rng, d->seed);
  for (int k = 0; k < d->n_terms; ++k) {
    const llg_term& T = d->terms[k];
    Term t;
    t.kind = T.kind;
    t.order = T.order;
    if (cudaMalloc((void**)&t.field, bytes) != cudaSuccess) {
      delete g;
      return fail("out of device memory");
    }
    g->terms.push_back(t);
    Term& tt = g->terms.back();
    if (T.kind == LLG_TERM_EXCHANGE) {
      std::vector<int> row, col;
      std::vector<double> val;
      if (build_csr(d, T, row, col, val)) {
        delete g;
        return -1;
      }
      tt.nnz = (int64_t)col.size();
      if (upload(&tt.row, row) != cudaSuccess || upload(&tt.col, col) != cudaSuccess ||
          upload(&tt.val, val) != cudaSuccess) {
        delete g;
        return fail("out of device memory (CSR)");
      }
      cusparseCreateCsr(&tt.A, 3 * (int64_t)n, 3 * (int64_t)n, tt.nnz, tt.row, tt.col, tt.val, CUSPARSE_INDEX_32I,
                        CUSPARSE_INDEX_32I, CUSPARSE_INDEX_BASE_ZERO, CUDA_R_64F);
      cusparseCreateDnVec(&tt.x, 3 * (int64_t)n, g->s, CUDA_R_64F);
      cusparseCreateDnVec(&tt.y, 3 * (int64_t)n, tt.field, CUDA_R_64F);
    } else if (T.kind == LLG_TERM_UNIAXIAL || T.kind == LLG_TERM_CUBIC) {
      const int na = T.kind == LLG_TERM_UNIAXIAL ? 3 : 9;
      std::vector<double> K(n), ax((size_t)na * n);
      for (int i = 0; i < n; ++i) {
        K[i] = T.K[i % nb];
        for (int a = 0; a < na; ++a) ax[(size_t)na * i + a] = T.axis[na * (i % nb) + a];
      }
      if (upload(&tt.K, K) != cudaSuccess || upload(&tt.axis, ax) != cudaSuccess) {
        delete g;
        return fail("out of device memory");
      }
    } else if (T.kind == LLG_TERM_APPLIED_FIELD) {
      const double* B = R.use_B ? R.B : T.B;
      for (int a = 0; a < 3; ++a) tt.B[a] = B[a];
      if (T.pulse != LLG_PULSE_STATIC) {
        delete g;
        return fail("time-dependent fields are not in this restatement");
      }
    } else {
      delete g;
      return fail("term kind not in this restatement");
    }
  }
  if (g->terms.empty()) {
    delete g;
    return fail("no terms");
  }
  *out = g;
  return 0;
}

__attribute__((visibility("default"))) int refgpu_set_state(void* h, const double* s) {
  RefGpu* g = static_cast<RefGpu*>(h);
  return cudaMemcpy(g->s, s, (size_t)g->n * 3 * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess ? 0 : -1;
}

__attribute__((visibility("default"))) int refgpu_get_state(void* h, double* s) {
  RefGpu* g = static_cast<RefGpu*>(h);
  cudaStreamSynchronize(g->stream);
  return cudaMemcpy(s, g->s, (size_t)g->n * 3 * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : -1;
}

// nsteps steps; *ms: their duration measured with CUDA events on the stream
__attribute__((visibility("default"))) int refgpu_run(void* h, int nsteps, float* ms) {
  RefGpu* g = static_cast<RefGpu*>(h);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, g->stream);
  for (int k = 0; k < nsteps; ++k) step(g);
  cudaEventRecord(b, g->stream);
  cudaError_t ce = cudaEventSynchronize(b);
  float t = 0.f;
  cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (ms) *ms = t;
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) return fail(std::string("CUDA: ") + cudaGetErrorString(ce));
  return 0;
}

__attribute__((visibility("default"))) void refgpu_destroy(void* h) { delete static_cast<RefGpu*>(h); }

}  // extern "C"
