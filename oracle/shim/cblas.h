// Stand-in for the CBLAS header: the oracle harness supplies cblas_daxpy as a
// plain loop (y[i] += a * x[i]) compiled without floating-point contraction.
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
void cblas_daxpy(int n, double a, const double* x, int incx, double* y, int incy);
#ifdef __cplusplus
}
#endif
