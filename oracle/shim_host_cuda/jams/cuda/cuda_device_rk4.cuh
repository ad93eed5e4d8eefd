// Stand-in for the reference's device-side RK4 template header, which
// cuda_llg_rk4_kernel.cuh includes but does not use (it needs nvstd::function
// from the CUDA toolkit).  Used only by oracle/ref_rk4_kernels.cc, the host
// build of the reference's RK4 kernels.
#pragma once
