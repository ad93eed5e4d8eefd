// Stand-in for LAPACKE: only the prototypes the reference's Mat3 header names.
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
void sgetrf_(const int* m, const int* n, float* a, const int* lda, int* ipiv, int* info);
void sgetri_(const int* n, float* a, const int* lda, const int* ipiv, float* work, const int* lwork, int* info);
void dgetrf_(const int* m, const int* n, double* a, const int* lda, int* ipiv, int* info);
void dgetri_(const int* n, double* a, const int* lda, const int* ipiv, double* work, const int* lwork, int* info);
#ifdef __cplusplus
}
#endif
