// The REFERENCE's RK4 device kernels compiled for the host, so that the
// reference's own RK4 arithmetic can pin the oracle's restatement and the
// GPU's RK4 forms.  TEST INFRASTRUCTURE ONLY, built into
// oracle/_ref/libjams_ref.so by oracle/Makefile.ref where the reference
// sources are present.
//
// Included from the reference tree, unmodified:
//   src/jams/solvers/cuda_llg_rk4_kernel.cuh   cuda_llg_rk4_kernel (k = rhs)
//   src/jams/solvers/cuda_rk4_base_kernel.cuh  cuda_spin_normalisation_kernel
//
// The CUDA qualifiers become nothing and the thread and block indices are
// host variables that the launch loops below step through, one "thread" at
// a time, for the 64-thread blocks of CudaRK4BaseSolver::run
// (src/jams/solvers/cuda_rk4_base.cu:91-97) and CUDALLGRK4Solver
// (src/jams/solvers/cuda_llg_rk4.cu:19-27).  rsqrt, a CUDA device function,
// is 1 / sqrt on the host (a correctly rounded square root and division;
// the device's reciprocal square root is within an ulp of it).  The
// device-side RK4 template header that cuda_llg_rk4_kernel.cuh also includes
// (cuda_device_rk4.cuh, unused by the kernel) is replaced by an empty
// stand-in in shim_host_cuda/.
#include <cmath>

namespace ref_host_cuda {
struct Index3 {
  unsigned x = 0, y = 0, z = 0;
};
}  // namespace ref_host_cuda

static ref_host_cuda::Index3 threadIdx, blockIdx, blockDim;

#define __global__
#define __device__
#define __host__
static inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }

#include "jams/solvers/cuda_llg_rk4_kernel.cuh"
#include "jams/solvers/cuda_rk4_base_kernel.cuh"

#undef __global__
#undef __device__
#undef __host__

namespace {
// a 1-D launch of `threads` threads in blocks of 64, run serially
template <class F>
void launch_1d(unsigned threads, F&& body) {
  blockDim.x = 64;
  const unsigned blocks = (threads + blockDim.x - 1) / blockDim.x;
  for (unsigned b = 0; b < blocks; ++b) {
    blockIdx.x = b;
    for (unsigned t = 0; t < blockDim.x; ++t) {
      threadIdx.x = t;
      body();
    }
  }
}
}  // namespace

// k = -gamma (S x H' + alpha S x (S x H')), H' = h / mu_s + noise: the
// reference's cuda_llg_rk4_kernel over all spins
void ref_host_llg_rk4_kernel(const double* s, double* k, const double* h, const double* noise, const double* gyro,
                             const double* mus, const double* alpha, unsigned n) {
  launch_1d(n, [&] { cuda_llg_rk4_kernel(s, k, h, noise, gyro, mus, alpha, n); });
}

// s = s_old + dt (k1 + 2 k2 + 2 k3 + k4) / 6, then s / |s| through rsqrt:
// the reference's cuda_spin_normalisation_kernel, which evaluates the same
// combination expression as cuda_rk4_combination_kernel and then the
// normalisation of cuda_normalise_spins_kernel (src/jams/cuda/cuda_spin_ops.cu:4-16)
void ref_host_rk4_combine_normalise(double* s, const double* s_old, const double* k1, const double* k2,
                                    const double* k3, const double* k4, double dt, unsigned n) {
  launch_1d(n, [&] { cuda_spin_normalisation_kernel(s, s_old, k1, k2, k3, k4, dt, n); });
}
