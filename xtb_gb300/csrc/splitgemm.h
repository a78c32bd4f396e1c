// Split-precision FP64 GEMM on the BF16 tensor cores (fixed-point digit slices, exact FP32
// chunk sums, FP64 recombination); see splitgemm.cu.
#pragma once
#include "common.cuh"

namespace xg {

// bytes of workspace for an M x N x K product with `slices` digits
size_t split_gemm_workspace(int M, int N, int K, int slices);
// C = alpha op(A) op(B) + beta C (row-major, op as in dgemm); slices 4..7 (5: ~2^-40 relative
// error per product term); dK / dN: optional device bounds on K and N.
void split_gemm(cudaStream_t st, bool ta, bool tb, int M, int N, int K, double alpha, const double* A, int lda,
                const double* B, int ldb, double beta, double* C, int ldc, int slices, void* work,
                const int* dK = nullptr, const int* dN = nullptr);

// Diagnostic: random M x K and K x N matrices (entries uniform(-1,1) 2^-e, e in [0, exp_range]),
// split and FP64 products.  out[0] max |dC| / (|A||B|), out[1] max |dC| / max |C|, out[2] split ms,
// out[3] FP64 ms, out[4] split TFLOP/s, out[5] FP64 TFLOP/s (2MNK flops, CUDA events).
void split_gemm_check(int M, int N, int K, int slices, unsigned seed, int exp_range, double* out);

}  // namespace xg
