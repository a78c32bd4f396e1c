// Dense FP64 linear algebra for the GFN2 SCC generalised eigenproblem on sm_103a.
//
// Replaces the reference's LAPACK sequence (src/mctc/lapack/eigensolve.F90:218-246:
// dpotrf once per single point, then dsygst + dsyevd + dtrsm per SCC iteration)
// with hand-written device kernels:
//   * Cholesky S = U^T U (blocked, right-looking) and X = U^-1 once per single point;
//   * A = X^T H X via FP64 GEMMs (the standard form of HC = SCe);
//   * Householder tridiagonalisation A = Q T Q^T in one cooperative kernel;
//   * all eigenvalues of T by Sturm-sequence bisection (one thread per eigenvalue);
//   * eigenvectors of T by inverse iteration with partial-pivoting tridiagonal LU;
//   * back-transformation Z = Q Y (one warp per eigenvector) and C = X Z.
// All matrices are row-major n x n with leading dimension lda.
#include <cooperative_groups.h>

#include "linalg.h"
#include "linalg_device.cuh"

namespace cg = cooperative_groups;

namespace xg {

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) k_dgemm(int M, int N, int K, double alpha, const double* __restrict__ A,
                                               int lda, const double* __restrict__ B, int ldb, double beta,
                                               double* __restrict__ C, int ldc, int flags, const int* __restrict__ dK,
                                               const int* __restrict__ dN) {
    dgemm_tile<TA, TB>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, flags, dK, dN, blockIdx.y * GBM,
                       blockIdx.x * GBN);
}

void dgemm(cudaStream_t st, bool ta, bool tb, int M, int N, int K, double alpha, const double* A, int lda,
           const double* B, int ldb, double beta, double* C, int ldc, int flags, const int* dK, const int* dN) {
    if (M <= 0 || N <= 0) return;
    dim3 grid(ceil_div(N, GBN), ceil_div(M, GBM));
    if (!ta && !tb) k_dgemm<false, false><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, flags, dK, dN);
    else if (ta && !tb) k_dgemm<true, false><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, flags, dK, dN);
    else if (!ta && tb) k_dgemm<false, true><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, flags, dK, dN);
    else k_dgemm<true, true><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, flags, dK, dN);
    XG_LAUNCH_CHECK();
}

// copy the lower triangle onto the upper one (after a GF_SYM product)
__global__ void k_mirror_lower(int n, double* __restrict__ C, int ldc) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    if (j > i) C[(size_t)i * ldc + j] = C[(size_t)j * ldc + i];
}

void mirror_lower(cudaStream_t st, int n, double* C, int ldc) {
    k_mirror_lower<<<ceil_div((long)n * n, 256), 256, 0, st>>>(n, C, ldc);
    XG_LAUNCH_CHECK();
}

// ------------------------------------------------------------------ Cholesky (upper)
constexpr int CNB = 32;

// Factor the b x b diagonal block at A[k0,k0] in shared memory; info[0] = first failing column + 1.
__global__ void k_potrf_diag(int n, double* A, int lda, int k0, int* info) {
    __shared__ double a[CNB][CNB + 1];
    const int b = min(CNB, n - k0);
    for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
        const int i = t / b, j = t % b;
        a[i][j] = A[(size_t)(k0 + i) * lda + k0 + j];
    }
    __syncthreads();
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int k = 0; k < b; ++k) {
        if (threadIdx.x == 0) {
            const double dkk = a[k][k];
            if (!(dkk > 0.0)) {
                if (bad == 0) bad = k0 + k + 1;
                a[k][k] = 1.0;
            } else {
                a[k][k] = sqrt(dkk);
            }
        }
        __syncthreads();
        const double dk = a[k][k];
        for (int j = k + 1 + threadIdx.x; j < b; j += blockDim.x) a[k][j] /= dk;
        __syncthreads();
        for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
            const int i = t / b, j = t % b;
            if (i > k && j >= i) a[i][j] -= a[k][i] * a[k][j];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
        const int i = t / b, j = t % b;
        A[(size_t)(k0 + i) * lda + k0 + j] = (j >= i) ? a[i][j] : 0.0;
    }
    if (threadIdx.x == 0 && bad && info[0] == 0) info[0] = bad;
}

// A12 := U11^-T A12 for the block row k0 (columns k0+b .. n-1); one thread per column.
__global__ void k_potrf_trsm(int n, double* A, int lda, int k0) {
    __shared__ double u[CNB][CNB + 1];
    const int b = min(CNB, n - k0);
    for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
        const int i = t / b, j = t % b;
        u[i][j] = A[(size_t)(k0 + i) * lda + k0 + j];
    }
    __syncthreads();
    const int j = k0 + b + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double x[CNB];
#pragma unroll
    for (int i = 0; i < CNB; ++i) {
        if (i < b) {
            double s = A[(size_t)(k0 + i) * lda + j];
            for (int k = 0; k < i; ++k) s -= u[k][i] * x[k];
            x[i] = s / u[i][i];
        }
    }
#pragma unroll
    for (int i = 0; i < CNB; ++i)
        if (i < b) A[(size_t)(k0 + i) * lda + j] = x[i];
}

__global__ void k_zero_lower(int n, double* A, int lda) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    if (j < i) A[(size_t)i * lda + j] = 0.0;
}

void potrf_upper(cudaStream_t st, int n, double* A, int lda, int* d_info) {
    XG_CUDA(cudaMemsetAsync(d_info, 0, sizeof(int), st));
    for (int k0 = 0; k0 < n; k0 += CNB) {
        const int b = std::min(CNB, n - k0);
        k_potrf_diag<<<1, 256, 0, st>>>(n, A, lda, k0, d_info);
        XG_LAUNCH_CHECK();
        const int m = n - k0 - b;
        if (m > 0) {
            k_potrf_trsm<<<ceil_div(m, 128), 128, 0, st>>>(n, A, lda, k0);
            XG_LAUNCH_CHECK();
            // A22 -= U12^T U12
            double* U12 = A + (size_t)k0 * lda + k0 + b;
            dgemm(st, true, false, m, m, b, -1.0, U12, lda, U12, lda, 1.0, A + (size_t)(k0 + b) * lda + k0 + b, lda);
        }
    }
    k_zero_lower<<<ceil_div((long)n * n, 256), 256, 0, st>>>(n, A, lda);
    XG_LAUNCH_CHECK();
}

// X = U^-1 (upper triangular), one warp per column j: x_i = -(sum_{k=i+1..j} U_ik x_k) / U_ii.
__global__ void k_trinv_upper(int n, const double* __restrict__ U, int ldu, double* __restrict__ X, int ldx) {
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (j >= n) return;
    for (int i = j + 1 + lane; i < n; i += 32) X[(size_t)i * ldx + j] = 0.0;
    if (lane == 0) X[(size_t)j * ldx + j] = 1.0 / U[(size_t)j * ldu + j];
    __syncwarp();
    for (int i = j - 1; i >= 0; --i) {
        const double* urow = U + (size_t)i * ldu;
        double s = 0.0;
        for (int k = i + 1 + lane; k <= j; k += 32) s = fma(urow[k], X[(size_t)k * ldx + j], s);
        s = warp_sum(s);
        if (lane == 0) X[(size_t)i * ldx + j] = -s / urow[i];
        __syncwarp();
    }
}

void trinv_upper(cudaStream_t st, int n, const double* U, int ldu, double* X, int ldx) {
    k_trinv_upper<<<ceil_div((long)n * 32, 256), 256, 0, st>>>(n, U, ldu, X, ldx);
    XG_LAUNCH_CHECK();
}

// ------------------------------------------------------------------ Householder tridiagonalisation
// A (symmetric, full storage) -> T = Q^T A Q with Q = H(0) H(1) ... H(n-3),
// H(k) = I - tau_k v_k v_k^T, v_k[0..k] = 0, v_k[k+1] = 1 (LAPACK dsytd2, lower).
// v_k is stored in row k of V; d (diag), e (sub-diagonal) of T.  A is destroyed.
//
// One pass over the trailing rows per column: the rank-2 update of step k-1 is
// applied lazily while the symmetric product p = tau A22 v of step k is formed,
// so A22 is read and written once per column.  The pivot row of step k misses
// only the update of step k-1, which every block adds on the fly from the
// pending vectors it keeps in shared memory.  p alternates between two buffers
// (p[0..n) and p[n..2n)), so one grid-wide barrier per column suffices: a block
// still reading p of step k cannot meet a writer of the same buffer before the
// barrier of step k+1.
__global__ void __launch_bounds__(256) k_sytrd(int n, double* __restrict__ A, int lda, double* __restrict__ V,
                                               double* __restrict__ tau, double* __restrict__ d, double* __restrict__ e,
                                               double* __restrict__ p2) {
    cg::grid_group grid = cg::this_grid();
    extern __shared__ double sm[];
    double* v = sm;            // [n] current reflector, offset k+1
    double* w = sm + n;        // [n]
    double* vp = sm + 2 * n;   // [n] pending update (previous step), offset k
    double* wp = sm + 3 * n;   // [n]
    double* red = sm + 4 * n;  // [32]
    const int lane = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    double tprev = 0.0;        // tau of the pending update (0: nothing pending)

    for (int k = 0; k < n - 2; ++k) {
        const int m = n - k - 1;
        double* p = p2 + (size_t)(k & 1) * n;
        const double* xk = A + (size_t)k * lda + k + 1;   // row k, pending update of step k-1 missing
        const bool pend = tprev != 0.0;
        const double v0 = pend ? vp[0] : 0.0, w0 = pend ? wp[0] : 0.0;
        double ss = 0.0;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            double xv = xk[i];
            if (pend) xv -= v0 * wp[i + 1] + w0 * vp[i + 1];
            v[i] = xv;
            if (i > 0) ss += xv * xv;
        }
        const double xnorm2 = block_sum(ss, red);
        const double alpha = v[0];
        double beta, tk, scale;
        if (xnorm2 == 0.0) {
            tk = 0.0;
            beta = alpha;
            scale = 0.0;
        } else {
            beta = -copysign(sqrt(alpha * alpha + xnorm2), alpha);
            tk = (beta - alpha) / beta;
            scale = 1.0 / (alpha - beta);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < m; i += blockDim.x) v[i] = (i == 0) ? 1.0 : v[i] * scale;
        __syncthreads();
        if (blockIdx.x == 0) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) V[(size_t)k * n + i] = (i <= k) ? 0.0 : v[i - k - 1];
            if (threadIdx.x == 0) {
                tau[k] = tk;
                d[k] = A[(size_t)k * lda + k] - 2.0 * v0 * w0;
                e[k] = beta;
            }
        }
        // rows k+1 .. n-1: apply the pending update of step k-1 (cols >= k+1) and form
        // p = tau A22 v
        for (int r = gwarp; r < m; r += nwarps) {
            double* arow = A + (size_t)(k + 1 + r) * lda + k + 1;
            const double vr = pend ? vp[r + 1] : 0.0, wr = pend ? wp[r + 1] : 0.0;
            double sdot = 0.0;
            for (int c = lane; c < m; c += 32) {
                double a = arow[c];
                if (pend) {
                    a -= vr * wp[c + 1] + wr * vp[c + 1];
                    arow[c] = a;
                }
                sdot = fma(a, v[c], sdot);
            }
            sdot = warp_sum(sdot);
            if (lane == 0) p[r] = tk * sdot;
        }
        grid.sync();
        // w = p - (tau/2)(p.v) v; it becomes the pending update (offset k+1)
        if (tk != 0.0) {
            double pv = 0.0;
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                const double pi = p[i];
                w[i] = pi;
                pv += pi * v[i];
            }
            pv = block_sum(pv, red);
            const double kk = -0.5 * tk * pv;
            for (int i = threadIdx.x; i < m; i += blockDim.x) w[i] += kk * v[i];
        }
        __syncthreads();
        if (tk != 0.0)
            for (int i = threadIdx.x; i < m; i += blockDim.x) { vp[i] = v[i]; wp[i] = w[i]; }
        tprev = tk;
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (n >= 3) {
            // rows n-2 and n-1 still carry the pending update of step n-3 (offset n-2)
            double a11 = A[(size_t)(n - 2) * lda + n - 2];
            double a21 = A[(size_t)(n - 1) * lda + n - 2];
            double a22 = A[(size_t)(n - 1) * lda + n - 1];
            if (tprev != 0.0) {
                a11 -= 2.0 * vp[0] * wp[0];
                a21 -= vp[1] * wp[0] + wp[1] * vp[0];
                a22 -= 2.0 * vp[1] * wp[1];
            }
            d[n - 2] = a11;
            e[n - 2] = a21;
            tau[n - 2] = 0.0;
            d[n - 1] = a22;
        } else if (n == 2) {
            d[0] = A[0];
            e[0] = A[(size_t)lda];
            tau[0] = 0.0;
            d[1] = A[(size_t)lda + 1];
        } else {
            d[n - 1] = A[(size_t)(n - 1) * lda + n - 1];
        }
        tau[n - 1] = 0.0;
    }
}

void sytrd(cudaStream_t st, int n, double* A, int lda, double* V, double* tau, double* d, double* e, double* p) {
    static int nsm = 0, maxblk = 0;
    const size_t smem = (size_t)(4 * n + 32) * sizeof(double);
    if (n <= 2) {
        // trivial: copy diagonal / off-diagonal
        k_sytrd<<<1, 256, smem, st>>>(n, A, lda, V, tau, d, e, p);
        XG_LAUNCH_CHECK();
        return;
    }
    int dev;
    XG_CUDA(cudaGetDevice(&dev));
    XG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    if (smem > 48 * 1024)
        XG_CUDA(cudaFuncSetAttribute(k_sytrd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxblk, k_sytrd, 256, smem));
    if (maxblk < 1) throw CudaError("sytrd: kernel does not fit on an SM");
    // enough warps to cover the rows, at most one co-resident wave
    int blocks = std::min(nsm * maxblk, std::max(1, ceil_div(n, 8)));
    void* args[] = {&n, &A, &lda, &V, &tau, &d, &e, &p};
    XG_CUDA(cudaLaunchCooperativeKernel((void*)k_sytrd, blocks, 256, args, smem, st));
    ++launch_counter();
}

// ------------------------------------------------------------------ bisection
// Number of eigenvalues of T below x, from the sign changes of the leading principal minors
// p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2}, p_{-1} = 1 (Sturm sequence, three-term form).
// Only one FMA per row sits on the dependent chain and no division is needed, which matters on
// a part whose FP64 divide is a long multi-instruction sequence.  A minor that comes out exactly
// zero is replaced by a tiny value of the sign opposite to its predecessor (the ratio p_i/p_{i-1}
// becomes a tiny negative number, as the pivmin rule of the ratio form makes it); the pair
// (p_i, p_{i-1}) is rescaled by an exact power of two whenever its larger exponent leaves
// [2^-400, 2^400], so neither overflows nor underflows.  Sign and exponent tests use integer
// operations on the bit pattern.  d and e2 are read from shared memory.
__device__ __forceinline__ int dexp_bits(double v) { return (__double2hiint(v) >> 20) & 0x7ff; }

__device__ int sturm_count(int n, const double* d, const double* e2, double x) {
    double pm = 1.0, p = d[0] - x;
    if (p == 0.0) p = -0x1p-600;
    int cnt = __double2hiint(p) < 0;
    for (int i = 1; i < n; ++i) {
        double pn = fma(d[i] - x, p, -e2[i - 1] * pm);
        if ((__double_as_longlong(pn) << 1) == 0) pn = -0x1p-600 * p;
        cnt += (__double2hiint(pn) ^ __double2hiint(p)) < 0;
        const int ex = max(dexp_bits(pn), dexp_bits(p));
        if (ex > 1023 + 400) { pn *= 0x1p-400; p *= 0x1p-400; }
        else if (ex < 1023 - 400) { pn *= 0x1p+400; p *= 0x1p+400; }
        pm = p;
        p = pn;
    }
    return cnt;
}

__global__ void k_tri_prep(int n, const double* __restrict__ d, const double* __restrict__ e, double* __restrict__ e2,
                           double* __restrict__ bounds) {
    // single block: e2 = e^2, Gershgorin bounds, pivmin, 1-norm
    double lo = 1e300, hi = -1e300, emax = 0.0, tn = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double el = (i > 0) ? fabs(e[i - 1]) : 0.0;
        const double er = (i < n - 1) ? fabs(e[i]) : 0.0;
        lo = fmin(lo, d[i] - el - er);
        hi = fmax(hi, d[i] + el + er);
        tn = fmax(tn, fabs(d[i]) + el + er);
        if (i < n - 1) {
            e2[i] = e[i] * e[i];
            emax = fmax(emax, e[i] * e[i]);
        }
    }
    // block min/max via shared reductions
    __shared__ double slo[32], shi[32], sem[32], stn[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o));
    }
    if (lane == 0) { slo[wid] = lo; shi[wid] = hi; sem[wid] = emax; stn[wid] = tn; }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) / 32;
        for (int k = 1; k < nw; ++k) {
            lo = fmin(lo, slo[k]); hi = fmax(hi, shi[k]); emax = fmax(emax, sem[k]); tn = fmax(tn, stn[k]);
        }
        lo = slo[0] < lo ? slo[0] : lo;
        const double span = fmax(hi - lo, 1e-300);
        bounds[0] = lo - 2.0 * 2.220446049250313e-16 * span - 1e-300;
        bounds[1] = hi + 2.0 * 2.220446049250313e-16 * span + 1e-300;
        bounds[2] = fmax(2.2250738585072014e-308, 2.2250738585072014e-308 * emax);   // pivmin
        bounds[3] = tn;                                                                // ||T||_inf
    }
}

// Eigenvalue j of T by bisection on Sturm counts, one thread per eigenvalue, to an
// absolute accuracy of 2 eps ||T|| (the accuracy inverse iteration needs).  One warp per
// block, so the eigenvalues spread over as many SMs as possible (the FP64 pipe of an SM is
// the limit); d and e^2 are staged in shared memory (dynamic, 2n doubles).
__global__ void __launch_bounds__(32) k_bisect(int n, const double* __restrict__ d, const double* __restrict__ e2,
                                               const double* __restrict__ bounds, double* __restrict__ w) {
    extern __shared__ double sde[];
    double* sd = sde;
    double* se = sde + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        sd[i] = d[i];
        se[i] = (i < n - 1) ? e2[i] : 0.0;
    }
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double lo = bounds[0], hi = bounds[1];
    const double atol = 2.0 * 2.220446049250313e-16 * fmax(bounds[3], 1e-300);
    for (int it = 0; it < 80; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (hi - lo <= atol || mid <= lo || mid >= hi) break;
        if (sturm_count(n, sd, se, mid) > j) hi = mid; else lo = mid;
    }
    w[j] = 0.5 * (lo + hi);
}

// ------------------------------------------------------------------ inverse iteration
// Eigenvector j of T for eigenvalue w[j]; output Y[i*n + j].  Scratch arrays are
// [i*n + j] so that the threads of a warp (consecutive j) access consecutive words.
__global__ void k_inviter(int n, const double* __restrict__ d, const double* __restrict__ e,
                          const double* __restrict__ w, const double* __restrict__ bounds, double* __restrict__ Y,
                          double* __restrict__ U1, double* __restrict__ U2, double* __restrict__ U3,
                          double* __restrict__ ML, unsigned char* __restrict__ piv, const int* __restrict__ ncol) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n || (ncol && j >= *ncol)) return;
    const double tnorm = fmax(bounds[3], 1e-300);
    const double eps = 2.220446049250313e-16;
    double lam = w[j];
    // separate exactly coincident eigenvalues so that their vectors differ
    if (j > 0) {
        int k = j;
        while (k > 0 && w[k - 1] >= w[k] - 10.0 * eps * tnorm) --k;
        lam += (double)(j - k) * 10.0 * eps * tnorm;
    }
    const double pert = eps * tnorm;
    auto at = [n, j](int i) { return (size_t)i * n + j; };
    if (n == 1) { Y[at(0)] = 1.0; return; }
    // LU with partial pivoting of T - lam I
    double w0 = d[0] - lam, w1 = e[0];
    for (int i = 0; i < n - 1; ++i) {
        const double sub = e[i];
        const double nd = d[i + 1] - lam;
        const double ns = (i + 1 < n - 1) ? e[i + 1] : 0.0;
        if (fabs(w0) >= fabs(sub)) {
            double u0 = w0;
            if (fabs(u0) < pert) u0 = copysign(pert, u0 == 0.0 ? 1.0 : u0);
            const double r0 = 1.0 / u0;
            const double m = sub * r0;
            U1[at(i)] = r0; U2[at(i)] = w1; U3[at(i)] = 0.0; ML[at(i)] = m; piv[at(i)] = 0;
            w0 = nd - m * w1;
            w1 = ns;
        } else {
            const double r0 = 1.0 / sub;
            const double m = w0 * r0;
            U1[at(i)] = r0; U2[at(i)] = nd; U3[at(i)] = ns; ML[at(i)] = m; piv[at(i)] = 1;
            w0 = w1 - m * nd;
            w1 = -m * ns;
        }
    }
    if (fabs(w0) < pert) w0 = copysign(pert, w0 == 0.0 ? 1.0 : w0);
    U1[at(n - 1)] = 1.0 / w0;   // U1 holds reciprocal pivots
    // start vector: deterministic pseudo-random
    uint32_t s = 0x9e3779b9u ^ (uint32_t)(j * 2654435761u);
    for (int i = 0; i < n; ++i) {
        s ^= s << 13; s ^= s >> 17; s ^= s << 5;
        Y[at(i)] = 0.5 + (double)(s & 0xffffff) / (double)0x1000000;
    }
    for (int iter = 0; iter < 3; ++iter) {
        // forward: apply row interchanges and multipliers
        for (int i = 0; i < n - 1; ++i) {
            double bi = Y[at(i)], bn = Y[at(i + 1)];
            if (piv[at(i)]) { const double t = bi; bi = bn; bn = t; Y[at(i)] = bi; }
            Y[at(i + 1)] = bn - ML[at(i)] * bi;
        }
        // back substitution
        double x2 = 0.0, x1 = Y[at(n - 1)] * U1[at(n - 1)];
        Y[at(n - 1)] = x1;
        double mx = fabs(x1);
        for (int i = n - 2; i >= 0; --i) {
            const double x = (Y[at(i)] - U2[at(i)] * x1 - U3[at(i)] * x2) * U1[at(i)];
            Y[at(i)] = x;
            x2 = x1;
            x1 = x;
            mx = fmax(mx, fabs(x));
        }
        // normalise (scale by max first to avoid overflow)
        const double inv = 1.0 / mx;
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) {
            const double x = Y[at(i)] * inv;
            Y[at(i)] = x;
            nrm += x * x;
        }
        const double sc = 1.0 / sqrt(nrm);
        for (int i = 0; i < n; ++i) Y[at(i)] *= sc;
    }
}

// Solve (T - lam_j I) x = b in place on column j of Y with the stored LU factors (one thread).
__device__ void tri_solve_col(int n, int j, const double* __restrict__ U1, const double* __restrict__ U2,
                              const double* __restrict__ U3, const double* __restrict__ ML,
                              const unsigned char* __restrict__ piv, double* __restrict__ Y) {
    auto at = [n, j](int i) { return (size_t)i * n + j; };
    for (int i = 0; i < n - 1; ++i) {
        double bi = Y[at(i)], bn = Y[at(i + 1)];
        if (piv[at(i)]) { const double t = bi; bi = bn; bn = t; Y[at(i)] = bi; }
        Y[at(i + 1)] = bn - ML[at(i)] * bi;
    }
    double x2 = 0.0, x1 = Y[at(n - 1)] * U1[at(n - 1)];
    Y[at(n - 1)] = x1;
    for (int i = n - 2; i >= 0; --i) {
        const double x = (Y[at(i)] - U2[at(i)] * x1 - U3[at(i)] * x2) * U1[at(i)];
        Y[at(i)] = x;
        x2 = x1;
        x1 = x;
    }
}

// Clusters of (near-)degenerate eigenvalues (gap < ctol*||T||): inverse iteration with
// modified Gram-Schmidt against the earlier members after every solve (as dstein does).
// One warp per cluster, started by its first member; members are processed in order.
__global__ void k_reorth(int n, const double* __restrict__ w, const double* __restrict__ bounds, double ctol,
                         double* __restrict__ Y, const double* __restrict__ U1, const double* __restrict__ U2,
                         const double* __restrict__ U3, const double* __restrict__ ML,
                         const unsigned char* __restrict__ piv, const int* __restrict__ ncol) {
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nc = ncol ? min(n, *ncol) : n;
    if (j >= nc) return;
    const double tol = ctol * fmax(bounds[3], 1e-300);
    if (j > 0 && w[j] - w[j - 1] < tol) return;          // not the first member
    int end = j + 1;
    while (end < nc && w[end] - w[end - 1] < tol) ++end;
    if (end - j < 2) return;
    for (int k = j + 1; k < end; ++k) {
        for (int rep = 0; rep < 3; ++rep) {
            if (rep > 0) {
                if (lane == 0) tri_solve_col(n, k, U1, U2, U3, ML, piv, Y);
                __syncwarp();
                double mx = 0.0;
                for (int r = lane; r < n; r += 32) mx = fmax(mx, fabs(Y[(size_t)r * n + k]));
                for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                const double inv = 1.0 / mx;
                for (int r = lane; r < n; r += 32) Y[(size_t)r * n + k] *= inv;
                __syncwarp();
            }
            for (int i = j; i < k; ++i) {
                double sdot = 0.0;
                for (int r = lane; r < n; r += 32) sdot += Y[(size_t)r * n + i] * Y[(size_t)r * n + k];
                sdot = warp_sum(sdot);
                for (int r = lane; r < n; r += 32) Y[(size_t)r * n + k] -= sdot * Y[(size_t)r * n + i];
                __syncwarp();
            }
            double nr = 0.0;
            for (int r = lane; r < n; r += 32) nr += Y[(size_t)r * n + k] * Y[(size_t)r * n + k];
            nr = warp_sum(nr);
            const double sc = 1.0 / sqrt(nr);
            for (int r = lane; r < n; r += 32) Y[(size_t)r * n + k] *= sc;
            __syncwarp();
        }
    }
}

void tridiag_eigvals(cudaStream_t st, int n, const double* d, const double* e, double* e2, double* bounds,
                     double* w) {
    k_tri_prep<<<1, 256, 0, st>>>(n, d, e, e2, bounds);
    XG_LAUNCH_CHECK();
    const size_t smem = 2 * (size_t)n * sizeof(double);
    if (smem > 48 * 1024)
        XG_CUDA(cudaFuncSetAttribute(k_bisect, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_bisect<<<ceil_div(n, 32), 32, smem, st>>>(n, d, e2, bounds, w);
    XG_LAUNCH_CHECK();
}

void tridiag_eigvecs(cudaStream_t st, int n, const double* d, const double* e, const double* bounds, const double* w,
                     double* Y, double* scratch, unsigned char* pivbuf, const int* ncol) {
    const size_t nn = (size_t)n * n;
    k_inviter<<<ceil_div(n, 64), 64, 0, st>>>(n, d, e, w, bounds, Y, scratch, scratch + nn, scratch + 2 * nn,
                                              scratch + 3 * nn, pivbuf, ncol);
    XG_LAUNCH_CHECK();
    k_reorth<<<ceil_div((long)n * 32, 128), 128, 0, st>>>(n, w, bounds, 1.0e-7, Y, scratch, scratch + nn,
                                                        scratch + 2 * nn, scratch + 3 * nn, pivbuf, ncol);
    XG_LAUNCH_CHECK();
}

// ------------------------------------------------------------------ back-transformation
// Zt[j][:] = Q * Y[:, j] for every eigenvector j (one warp per eigenvector, vector staged in shared memory).
__global__ void k_ormtr(int n, const double* __restrict__ V, const double* __restrict__ tau,
                        const double* __restrict__ Y, double* __restrict__ Zt, const int* __restrict__ ncol) {
    extern __shared__ double sm[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const int j = blockIdx.x * wpb + wib;
    if (j >= n || (ncol && j >= *ncol)) return;
    double* y = sm + (size_t)wib * n;
    for (int i = lane; i < n; i += 32) y[i] = Y[(size_t)i * n + j];
    __syncwarp();
    for (int k = n - 3; k >= 0; --k) {
        const double t = tau[k];
        if (t == 0.0) continue;
        const double* vk = V + (size_t)k * n;
        double s = 0.0;
        for (int i = k + 1 + lane; i < n; i += 32) s = fma(vk[i], y[i], s);
        s = warp_sum(s) * t;
        for (int i = k + 1 + lane; i < n; i += 32) y[i] -= s * vk[i];
        __syncwarp();
    }
    for (int i = lane; i < n; i += 32) Zt[(size_t)j * n + i] = y[i];
}

void ormtr(cudaStream_t st, int n, const double* V, const double* tau, const double* Y, double* Zt, const int* ncol) {
    int wpb = 4;
    size_t smem = (size_t)wpb * n * sizeof(double);
    while (wpb > 1 && smem > 200 * 1024) { wpb >>= 1; smem = (size_t)wpb * n * sizeof(double); }
    if (smem > 48 * 1024) XG_CUDA(cudaFuncSetAttribute(k_ormtr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_ormtr<<<ceil_div(n, wpb), wpb * 32, smem, st>>>(n, V, tau, Y, Zt, ncol);
    XG_LAUNCH_CHECK();
}

}  // namespace xg

namespace xg {
// FP64 FMA throughput probe: 8 independent chains per thread, all SMs busy.
__global__ void k_fp64_probe(int iters, double* out) {
    double a[8];
    const double b = 1.0000000001, c = 1e-12;
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-3 + k;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 12345.678) out[0] = s;   // keep the chains alive
}

double fp64_peak_tflops() {
    int dev = 0, nsm = 0;
    XG_CUDA(cudaGetDevice(&dev));
    XG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    double* d = nullptr;
    XG_CUDA(cudaMalloc(&d, sizeof(double)));
    const int blocks = nsm * 8, threads = 256, iters = 1 << 14;
    cudaEvent_t e0, e1;
    XG_CUDA(cudaEventCreate(&e0));
    XG_CUDA(cudaEventCreate(&e1));
    k_fp64_probe<<<blocks, threads>>>(iters, d);   // warm-up
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        XG_CUDA(cudaEventRecord(e0));
        k_fp64_probe<<<blocks, threads>>>(iters, d);
        XG_CUDA(cudaEventRecord(e1));
        XG_CUDA(cudaEventSynchronize(e1));
        float ms;
        XG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        best = std::min(best, ms);
    }
    XG_CUDA(cudaEventDestroy(e0));
    XG_CUDA(cudaEventDestroy(e1));
    XG_CUDA(cudaFree(d));
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    return flops / (best * 1e-3) / 1e12;
}
}  // namespace xg
