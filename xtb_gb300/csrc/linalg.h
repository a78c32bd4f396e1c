// Host-side launchers of the FP64 dense linear algebra kernels (row-major storage).
#pragma once
#include <algorithm>

#include "common.cuh"

namespace xg {

// structure flags of dgemm
constexpr int GF_B_UPPER = 1, GF_A_LOWER = 2, GF_A_UPPER = 4, GF_SYM = 8, GF_SYM_UP = 16;
// C = alpha op(A) op(B) + beta C (see linalg.cu for the flags; dK / dN optional device bounds)
void dgemm(cudaStream_t st, bool ta, bool tb, int M, int N, int K, double alpha, const double* A, int lda,
           const double* B, int ldb, double beta, double* C, int ldc, int flags = 0, const int* dK = nullptr,
           const int* dN = nullptr);
// copy the lower triangle of C onto its upper triangle
void mirror_lower(cudaStream_t st, int n, double* C, int ldc);
// C <- C + C^T
void sym_add(cudaStream_t st, int n, double* C, int ldc);
// A = U^T U, U upper (lower triangle zeroed); d_info[0] = failing column + 1 or 0
void potrf_upper(cudaStream_t st, int n, double* A, int lda, int* d_info);
// X = U^-1
void trinv_upper(cudaStream_t st, int n, const double* U, int ldu, double* X, int ldx);
// Householder reduction to tridiagonal form (A destroyed); V[n*n], tau[n], d[n], e[n]; p[2n] scratch
// Householder tridiagonalisation of the symmetric n x n matrix A (one cooperative launch).
// p: sytrd_workspace(n) doubles of device scratch.
constexpr int SYTRD_SLOTS = 256;   // most blocks of the cooperative tridiagonalisation
// the upper-triangle form (4/3 n^3 flops) keeps three A x buffers and three per-column scalar
// arrays (6n doubles) after the row form's 2n + 2 SYTRD_SLOTS
inline size_t sytrd_workspace(int n) { return 8 * (size_t)n + 2 * (size_t)SYTRD_SLOTS; }
void sytrd(cudaStream_t st, int n, double* A, int lda, double* V, double* tau, double* d, double* e, double* p);
// the same with the form chosen: 0 the row-by-row form, 1 the upper-triangle form (when its
// shared memory fits), -1 by the device's measured threshold (tune.h)
// max_blocks > 0 caps the cooperative grid (so that concurrent single points can share the SMs)
void sytrd_form(cudaStream_t st, int n, double* A, int lda, double* V, double* tau, double* d, double* e, double* p,
                int form, int max_blocks = 0);
// eigenvalues of the tridiagonal (d, e): w[n] ascending; e2: n, bounds: 4.  With 0 < k < n only
// the lowest k (each is bisected on its own, so they equal those of the full call) and
// w[k..n) = 1e300.
void tridiag_eigvals(cudaStream_t st, int n, const double* d, const double* e, double* e2, double* bounds, double* w,
                     int k = -1);
// after tridiag_eigvals(..., k) and the Fermi smearing (scal = {entropy, e_fermi_a, e_fermi_b},
// energies in the units of bkt): gate[0] = 1 and the levels k..n-1 bisected when the k-th level
// lies less than 60 kT above a Fermi level, else gate[0] = 0 and nothing more
void tridiag_eigvals_rest(cudaStream_t st, int n, const double* d, const double* e2, const double* bounds, double* w,
                          int k, const double* scal, double bkt, int* gate);
// eigenvectors j < *ncol (all if ncol is null): Y[i*n+j] = component i of vector j.
// scratch: 4*n*n doubles, pivbuf: n*n bytes
void tridiag_eigvecs(cudaStream_t st, int n, const double* d, const double* e, const double* bounds, const double* w,
                     double* Y, double* scratch, unsigned char* pivbuf, const int* ncol);
// Zt[j][:] = Q Y[:, j] for j < *ncol (all if null)
void ormtr(cudaStream_t st, int n, const double* V, const double* tau, const double* Y, double* Zt,
           const int* ncol = nullptr);
// Y[:, j] = Q Y[:, j] in place for j < *ncol (all if null), Q = H(0) ... H(n-3): compact-WY blocks
// of 128 reflectors (FP64: every block on column strips in one launch; split precision: two
// tensor-core GEMMs per block); work: ormtr_workspace(n) doubles
size_t ormtr_workspace(int n);
// the same product, one warp per vector, in place (better below a few thousand AOs)
void ormtr_inplace(cudaStream_t st, int n, const double* V, const double* tau, double* Y, const int* ncol);
// slices > 0: the two large products per block as split-precision tensor-core GEMMs (split_work:
// split_gemm_workspace(n, n, n, slices) bytes)
void ormtr_blocked(cudaStream_t st, int n, const double* V, const double* tau, double* Y, const int* ncol,
                   double* work, int slices = 0, void* split_work = nullptr);
// measured FP64 throughput of the current device (TFLOP/s): the largest of two FMA probes and
// the FP64 GEMM at 4096^3; fp64_peak_detail gives the three figures of the last measurement
double fp64_peak_tflops();
void fp64_peak_detail(double* out);
// dependent-operation latency in cycles: [0] FP64 FMA, [1] FP64 add, [2] FP64 multiply,
// [3] FP64 divide, [4] FP32 FMA
void fp64_latency_cycles(double* cycles);
// Largest error of the fast FP64 reciprocal in ulps (out[0]) over out[1] checked values.
void reciprocal_check(double* out);

}  // namespace xg
