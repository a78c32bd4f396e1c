// Host-side launchers of the FP64 dense linear algebra kernels (row-major storage).
#pragma once
#include <algorithm>

#include "common.cuh"

namespace xg {

// C = alpha op(A) op(B) + beta C
void dgemm(cudaStream_t st, bool ta, bool tb, int M, int N, int K, double alpha, const double* A, int lda,
           const double* B, int ldb, double beta, double* C, int ldc);
// A = U^T U, U upper (lower triangle zeroed); d_info[0] = failing column + 1 or 0
void potrf_upper(cudaStream_t st, int n, double* A, int lda, int* d_info);
// X = U^-1
void trinv_upper(cudaStream_t st, int n, const double* U, int ldu, double* X, int ldx);
// Householder reduction to tridiagonal form (A destroyed); V[n*n], tau[n], d[n], e[n], p[n] scratch
void sytrd(cudaStream_t st, int n, double* A, int lda, double* V, double* tau, double* d, double* e, double* p);
// eigenpairs of the tridiagonal (d, e): w[n] ascending, Y[i*n+j] = component i of vector j.
// scratch: 4*n*n doubles, pivbuf: n*n bytes, e2: n, bounds: 4
void tridiag_eig(cudaStream_t st, int n, const double* d, const double* e, double* e2, double* bounds, double* w,
                 double* Y, double* scratch, unsigned char* pivbuf);
// Zt[j][:] = Q Y[:, j]
void ormtr(cudaStream_t st, int n, const double* V, const double* tau, const double* Y, double* Zt);
// measured FP64 FMA throughput of the current device (TFLOP/s)
double fp64_peak_tflops();

}  // namespace xg
