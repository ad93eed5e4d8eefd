// Magnetisation of a spin array that already lives on the device, computed
// without allocating any memory.
//
// Who needs it: code that must not call cudaMalloc/cudaFree at the moment it
// wants the magnetisation - a host loop that must not synchronise the device
// (cudaMalloc and cudaFree can), or a caller whose device memory is owned by
// an external pool or arena that forbids other allocations.  The regular
// path (llg_observables) keeps its reduction partials in memory the handle
// allocated; this entry point uses the same two-pass block reduction with
// its partials in a fixed, file-scope device array instead.
//
// Scratch: kNoAllocMaxBlocks x 4 doubles (32 KiB) of device memory, held by
// every GPU that loads this library until the process exits.  Every call on
// a device shares it and it keeps the previous call's contents; the first
// pass writes every slot the second pass reads, so nothing needs clearing.
// Two calls whose kernels overlap on the GPU (different streams without
// ordering) race on the array and give wrong results.  The array's device
// address is looked up once per device and kept: a cudaDeviceReset after the
// first call on a device is not supported (the reloaded module may put the
// array elsewhere).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/jams_llg.h"

namespace jams_llg {
void set_thread_error(const char* msg);  // llg_host.cu
}

namespace {

constexpr int kNoAllocBlock = 256;
constexpr int kNoAllocMaxBlocks = 1024;
constexpr int64_t kNoAllocMaxSpins = (int64_t)1 << 30;
constexpr int kNoAllocMaxBasis = 4;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks * 4];

struct Mus {
  double v[kNoAllocMaxBasis];
};

// pass 1: grid-stride sums of mu_s S (3) and mu_s per block, fixed tree order
__global__ void __launch_bounds__(kNoAllocBlock) noalloc_partials(const double* __restrict__ s, int64_t n, int nb,
                                                                  Mus mus, double* __restrict__ partials) {
  __shared__ double red[4][kNoAllocBlock];
  double q[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * kNoAllocBlock + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNoAllocBlock) {
    const double mu = mus.v[i % nb];
    q[0] += mu * s[3 * i];
    q[1] += mu * s[3 * i + 1];
    q[2] += mu * s[3 * i + 2];
    q[3] += mu;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = q[k];
  __syncthreads();
  for (int w = kNoAllocBlock / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
#pragma unroll
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) partials[blockIdx.x * 4 + threadIdx.x] = red[threadIdx.x][0];
}

// pass 2: one block adds the partials of the blocks used, writes m4
__global__ void __launch_bounds__(kNoAllocBlock) noalloc_finish(const double* __restrict__ partials, int nblocks,
                                                                double* __restrict__ m4) {
  __shared__ double red[4][kNoAllocBlock];
  double q[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblocks; b += kNoAllocBlock) {
#pragma unroll
    for (int k = 0; k < 4; ++k) q[k] += partials[b * 4 + k];
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = q[k];
  __syncthreads();
  for (int w = kNoAllocBlock / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
#pragma unroll
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double mx = red[0][0], my = red[1][0], mz = red[2][0], ms = red[3][0];
    m4[0] = mx / ms;
    m4[1] = my / ms;
    m4[2] = mz / ms;
    m4[3] = sqrt(mx * mx + my * my + mz * mz) / ms;
  }
}

std::mutex g_setup_mutex;
double* g_scratch_ptr[kNoAllocMaxDevices] = {};

int fail(int code, const char* msg) {
  jams_llg::set_thread_error(msg);
  return code;
}

}  // namespace

extern "C" int llg_magnetisation_noalloc(const double* spins_dev, int64_t n_spins, int32_t nb, const double* mus,
                                         double* m4_dev, void* cuda_stream) {
  if (!spins_dev || !m4_dev || !mus) return fail(LLG_ERR_BAD_DESC, "llg_magnetisation_noalloc: null pointer");
  if (nb < 1 || nb > kNoAllocMaxBasis)
    return fail(LLG_ERR_BAD_DESC, "llg_magnetisation_noalloc: nb must be in [1, 4]");
  if (n_spins < 1 || n_spins > kNoAllocMaxSpins || n_spins % nb != 0) {
    char buf[160];
    snprintf(buf, sizeof buf,
             "llg_magnetisation_noalloc: n_spins = %lld outside [1, %lld] or not a multiple of nb = %d",
             (long long)n_spins, (long long)kNoAllocMaxSpins, nb);
    return fail(LLG_ERR_BAD_DESC, buf);
  }
  Mus m{};
  for (int b = 0; b < nb; ++b) {
    if (!(std::isfinite(mus[b]) && mus[b] > 0.0))
      return fail(LLG_ERR_BAD_DESC, "llg_magnetisation_noalloc: mu_s must be positive and finite");
    m.v[b] = mus[b];
  }
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return fail(LLG_ERR_CUDA, cudaGetErrorString(ce));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(LLG_ERR_NO_DEVICE, "llg_magnetisation_noalloc: device ordinal");
  double* scratch = nullptr;
  {
    // set-up, once per device, with that device current: the device address
    // of the file-scope array (in host code its name is only a stand-in)
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      ce = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (ce != cudaSuccess) return fail(LLG_ERR_CUDA, cudaGetErrorString(ce));
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  const int64_t want = (n_spins + kNoAllocBlock - 1) / kNoAllocBlock;
  const int nblocks = (int)(want < kNoAllocMaxBlocks ? want : kNoAllocMaxBlocks);
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  // an error left pending by earlier, unrelated work is cleared here, so that
  // the check after the launches reports only these launches (an error that
  // corrupted the context persists and is reported there)
  (void)cudaGetLastError();
  noalloc_partials<<<nblocks, kNoAllocBlock, 0, st>>>(spins_dev, n_spins, nb, m, scratch);
  noalloc_finish<<<1, kNoAllocBlock, 0, st>>>(scratch, nblocks, m4_dev);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return fail(LLG_ERR_CUDA, cudaGetErrorString(ce));
  return 0;
}
