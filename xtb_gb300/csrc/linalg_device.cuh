// Device-side FP64 GEMM tile shared by the per-molecule launchers and the batched engine.
#pragma once
#include "linalg.h"

namespace xg {

// ------------------------------------------------------------------ GEMM
constexpr int GBM = 64, GBN = 64, GBK = 16;

// C[M,N] = alpha * op(A) * op(B) + beta * C.
// op(A)[i,k] = TA ? A[k*lda+i] : A[i*lda+k];  op(B)[k,j] = TB ? B[j*ldb+k] : B[k*ldb+j].
// Structure flags skip work that is known to be zero or redundant:
//   GF_B_UPPER  op(B)[k,j] = 0 for k > j      (k < j0 + 64 per tile)
//   GF_A_LOWER  op(A)[i,k] = 0 for k > i      (k < i0 + 64 per tile)
//   GF_A_UPPER  op(A)[i,k] = 0 for k < i      (k >= i0 per tile)
//   GF_SYM      C symmetric: only tiles touching the lower triangle are computed (mirror afterwards)
// dK / dN (optional, device): K and N limited to *dK / *dN at run time.
// One 64x64 tile (i0, j0) of the product, computed by a 256-thread block.
template <bool TA, bool TB>
__device__ void dgemm_tile(int M, int N, int K, double alpha, const double* __restrict__ A, int lda,
                           const double* __restrict__ B, int ldb, double beta, double* __restrict__ C, int ldc,
                           int flags, const int* __restrict__ dK, const int* __restrict__ dN, int i0, int j0) {
    __shared__ double As[2][GBK][GBM + 1];
    __shared__ double Bs[2][GBK][GBN + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    if (dN) N = min(N, *dN);
    if (j0 >= N) return;
    if ((flags & GF_SYM) && j0 >= i0 + GBM) return;
    if (dK) K = min(K, *dK);
    int kbeg = 0, kend = K;
    if (flags & GF_B_UPPER) kend = min(kend, j0 + GBN);
    if (flags & GF_A_LOWER) kend = min(kend, i0 + GBM);
    if (flags & GF_A_UPPER) kbeg = (i0 / GBK) * GBK;
    double acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = 0.0;

    auto load = [&](int buf, int k0) {
#pragma unroll
        for (int s = 0; s < (GBM * GBK) / 256; ++s) {
            const int t = threadIdx.x + s * 256;
            int ii, kk;
            if (TA) { ii = t % GBM; kk = t / GBM; } else { kk = t % GBK; ii = t / GBK; }
            const int gi = i0 + ii, gk = k0 + kk;
            double v = 0.0;
            if (gi < M && gk < kend) v = TA ? A[(size_t)gk * lda + gi] : A[(size_t)gi * lda + gk];
            As[buf][kk][ii] = v;
        }
#pragma unroll
        for (int s = 0; s < (GBN * GBK) / 256; ++s) {
            const int t = threadIdx.x + s * 256;
            int jj, kk;
            if (TB) { kk = t % GBK; jj = t / GBK; } else { jj = t % GBN; kk = t / GBN; }
            const int gj = j0 + jj, gk = k0 + kk;
            double v = 0.0;
            if (gj < N && gk < kend) v = TB ? B[(size_t)gj * ldb + gk] : B[(size_t)gk * ldb + gj];
            Bs[buf][kk][jj] = v;
        }
    };

    int buf = 0;
    if (kbeg < kend) load(0, kbeg);
    __syncthreads();
    for (int k0 = kbeg; k0 < kend; k0 += GBK) {
        if (k0 + GBK < kend) load(buf ^ 1, k0 + GBK);
#pragma unroll
        for (int kk = 0; kk < GBK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[buf][kk][ty + 16 * r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[buf][kk][tx + 16 * c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
        buf ^= 1;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int i = i0 + ty + 16 * r;
        if (i >= M) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int j = j0 + tx + 16 * c;
            if (j >= N) continue;
            double v = alpha * acc[r][c];
            if (beta != 0.0) v += beta * C[(size_t)i * ldc + j];
            C[(size_t)i * ldc + j] = v;
        }
    }
}

// Whole product by one 256-thread block (tiles in sequence); used for small per-molecule matrices.
template <bool TA, bool TB>
__device__ void cta_dgemm(int M, int N, int K, double alpha, const double* A, int lda, const double* B, int ldb,
                          double beta, double* C, int ldc, int flags, const int* dK, const int* dN) {
    for (int i0 = 0; i0 < M; i0 += GBM)
        for (int j0 = 0; j0 < N; j0 += GBN) {
            dgemm_tile<TA, TB>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, flags, dK, dN, i0, j0);
            __syncthreads();
        }
}

}  // namespace xg
