// Device-side FP64 GEMM tile shared by the per-molecule launchers and the batched engine.
#pragma once
#include <cooperative_groups.h>

#include "linalg.h"

namespace cg = cooperative_groups;

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
//   GF_SYM_UP   C symmetric and only its upper triangle wanted: tiles touching the upper triangle
// dK / dN (optional, device): K and N limited to *dK / *dN at run time.
// One TB x TB tile (i0, j0) of the product (TB = 64 or 32), computed by a 256-thread block: thread
// (tx, ty) owns rows ty + 16 r and columns tx + 16 c, r, c < TB / 16.
template <bool TA, bool TB, int TBS = GBM>
__device__ inline void dgemm_tile(int M, int N, int K, double alpha, const double* __restrict__ A, int lda,
                           const double* __restrict__ B, int ldb, double beta, double* __restrict__ C, int ldc,
                           int flags, const int* __restrict__ dK, const int* __restrict__ dN, int i0, int j0,
                           double* smem) {
    constexpr int TM = TBS, TN = TBS, R = TBS / 16;
    double (*As)[GBK][TM + 1] = reinterpret_cast<double (*)[GBK][TM + 1]>(smem);
    double (*Bs)[GBK][TN + 1] = reinterpret_cast<double (*)[GBK][TN + 1]>(smem + 2 * GBK * (TM + 1));
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    if (dN) N = min(N, *dN);
    if (j0 >= N) return;
    if ((flags & GF_SYM) && j0 >= i0 + TM) return;
    if ((flags & GF_SYM_UP) && i0 >= j0 + TN) return;
    if (dK) K = min(K, *dK);
    int kbeg = 0, kend = K;
    if (flags & GF_B_UPPER) kend = min(kend, j0 + TN);
    if (flags & GF_A_LOWER) kend = min(kend, i0 + TM);
    if (flags & GF_A_UPPER) kbeg = (i0 / GBK) * GBK;
    double acc[R][R];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < R; ++c) acc[r][c] = 0.0;

    auto load = [&](int buf, int k0) {
#pragma unroll
        for (int s = 0; s < (TM * GBK) / 256; ++s) {
            const int t = threadIdx.x + s * 256;
            int ii, kk;
            if (TA) { ii = t % TM; kk = t / TM; } else { kk = t % GBK; ii = t / GBK; }
            const int gi = i0 + ii, gk = k0 + kk;
            double v = 0.0;
            if (gi < M && gk < kend) v = TA ? A[(size_t)gk * lda + gi] : A[(size_t)gi * lda + gk];
            As[buf][kk][ii] = v;
        }
#pragma unroll
        for (int s = 0; s < (TN * GBK) / 256; ++s) {
            const int t = threadIdx.x + s * 256;
            int jj, kk;
            if (TB) { kk = t % GBK; jj = t / GBK; } else { jj = t % TN; kk = t / TN; }
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
            double a[R], b[R];
#pragma unroll
            for (int r = 0; r < R; ++r) a[r] = As[buf][kk][ty + 16 * r];
#pragma unroll
            for (int c = 0; c < R; ++c) b[c] = Bs[buf][kk][tx + 16 * c];
#pragma unroll
            for (int r = 0; r < R; ++r)
#pragma unroll
                for (int c = 0; c < R; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
        buf ^= 1;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int i = i0 + ty + 16 * r;
        if (i >= M) continue;
#pragma unroll
        for (int c = 0; c < R; ++c) {
            const int j = j0 + tx + 16 * c;
            if (j >= N) continue;
            double v = alpha * acc[r][c];
            if (beta != 0.0) v += beta * C[(size_t)i * ldc + j];
            C[(size_t)i * ldc + j] = v;
        }
    }
}

// shared memory of one GEMM tile (doubles)
constexpr int GEMM_SMEM = 2 * GBK * (GBM + 1) + 2 * GBK * (GBN + 1);

// Whole product by one 256-thread block (tiles in sequence); used for small per-molecule matrices.
// 32 x 32 tiles: for the few-hundred-AO matrices of a batch, 64 x 64 tiles would compute up to
// 2.5x the needed products on padding (the FP64 pipe is the limit there).
// smem: GEMM_SMEM doubles of shared memory.
template <bool TA, bool TB>
__device__ inline void cta_dgemm(int M, int N, int K, double alpha, const double* A, int lda, const double* B, int ldb,
                          double beta, double* C, int ldc, int flags, const int* dK, const int* dN, double* smem) {
    constexpr int T = 32;
    for (int i0 = 0; i0 < M; i0 += T)
        for (int j0 = 0; j0 < N; j0 += T) {
            dgemm_tile<TA, TB, T>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, flags, dK, dN, i0, j0, smem);
            __syncthreads();
        }
}

// X = U^-1 (upper triangular), one warp per column j: x_i = -(sum_{k=i+1..j} U_ik x_k) / U_ii.
__device__ inline void d_trinv_col(int n, const double* __restrict__ U, int ldu, double* __restrict__ X, int ldx, int j,
                            int lane) {
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
// barrier of step k+1.  The grid form also leaves each block's share of p.v in
// two alternating slot arrays (after p: 2 x SYTRD_SLOTS doubles), which every block
// sums in the same order after the barrier.
//
// Each warp streams its row in chunks of 32 x RT elements with the next chunk's loads
// issued before the current chunk is processed: the trailing matrix lives in L2, and a
// row pass that waits for every load is bound by L2 latency, not by the FP64 pipe.
//
// CTA = true: the whole reduction by one thread block (__syncthreads for the barrier),
// used by the batched engine; CTA = false: all blocks of a cooperative launch (at most
// SYTRD_SLOTS blocks).  sm: 4n + 68 doubles of shared memory (4n + 32 for CTA = true
// with at most 32 warps).

// Sum of red[0..nw) in four interleaved chains (nw a multiple of 4; FP64 additions have a
// long dependent latency, so a serial sum over the warps of a block is slow).
__device__ __forceinline__ double sum_slots4(const double* red, int nw) {
    double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
    for (int k = 0; k < nw; k += 4) {
        t0 += red[k];
        t1 += red[k + 1];
        t2 += red[k + 2];
        t3 += red[k + 3];
    }
    return (t0 + t1) + (t2 + t3);
}

__device__ __forceinline__ double block_sum4(double v, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    if (threadIdx.x < 4 && nw + (int)threadIdx.x < ((nw + 3) & ~3)) red[nw + threadIdx.x] = 0.0;
    __syncthreads();
    return sum_slots4(red, (nw + 3) & ~3);
}

template <bool CTA, bool PREFETCH = false>
__device__ inline void d_sytrd(int n, double* __restrict__ A, int lda, double* __restrict__ V, double* __restrict__ tau,
                               double* __restrict__ d, double* __restrict__ e, double* __restrict__ p2, double* sm) {
    constexpr int RT = CTA ? 2 : 8;   // chunk of a row pass: RT elements per lane
    // two sets of (reflector v, update vector w), offset k+1 at step k: set `cur` holds step
    // k's, the other the pending update of step k-1; the roles swap every column, and the
    // pending set's v buffer receives the next pivot row once step k's row pass is done
    double* red = sm + 4 * n;  // [36] block reductions
    double* wred = red + 36;   // [32] per-warp p.v of the grid form
    double* slots = p2 + 2 * (size_t)n;   // grid form: [2][SYTRD_SLOTS] per-block p.v
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    // grid form: consecutive rows go to consecutive blocks (warp w of block b takes rows
    // w*G + b (mod G*warps)), so that every SM's FP64 pipe gets a share of the trailing rows
    // even when there are fewer rows than warps
    const int gwarp = CTA ? wid : (int)(wid * gridDim.x + blockIdx.x);
    const int nwarps = CTA ? (int)(blockDim.x >> 5) : (int)((gridDim.x * blockDim.x) >> 5);
    const bool lead = CTA || blockIdx.x == 0;

    // Householder reflector of step k from row k's trailing part, already in x[0..m) with the
    // pending update (pv, pw: step k-1's v, w; ptau = 0 when there is none) still missing.
    // Leaves v_k in x and returns tau_k; the lead block stores v_k, tau_k, d_k, e_k.
    auto reflector = [&](int k, double* x, const double* pv, const double* pw, double ptau) -> double {
        const int m = n - k - 1;
        const bool pend = ptau != 0.0;
        const double v0 = pend ? pv[0] : 0.0, w0 = pend ? pw[0] : 0.0;
        double ss = 0.0;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            double xv = x[i];
            if (pend) xv -= v0 * pw[i + 1] + w0 * pv[i + 1];
            x[i] = xv;
            if (i > 0) ss += xv * xv;
        }
        const double xnorm2 = block_sum4(ss, red);
        const double alpha = x[0];
        double beta, tk, scale;
        if (xnorm2 == 0.0) {
            tk = 0.0;
            beta = alpha;
            scale = 0.0;
        } else {
            beta = -copysign(sqrt(alpha * alpha + xnorm2), alpha);
            tk = (beta - alpha) * rcp_fast(beta);
            scale = rcp_fast(alpha - beta);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < m; i += blockDim.x) x[i] = (i == 0) ? 1.0 : x[i] * scale;
        __syncthreads();
        if (lead) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) V[(size_t)k * n + i] = (i <= k) ? 0.0 : x[i - k - 1];
            if (threadIdx.x == 0) {
                tau[k] = tk;
                d[k] = A[(size_t)k * lda + k] - 2.0 * v0 * w0;
                e[k] = beta;
            }
        }
        return tk;
    };

    int cur = 0;
    double tprev = 0.0;        // tau of the pending update (0: nothing pending)
    double tk = 0.0;
    // PREFETCH: the first chunk of this warp's first row of the coming step is loaded right
    // after the barrier, so that its L2 latency overlaps the reflector (the row is final once
    // the barrier is passed); it costs RT registers held across the reflector
    double pre[RT];
    bool pre_ok = false;
    if (n > 2) {
        for (int i = threadIdx.x; i < n - 1; i += blockDim.x) sm[i] = A[i + 1];
        tk = reflector(0, sm, nullptr, nullptr, 0.0);
    }
    for (int k = 0; k < n - 2; ++k) {
        const int m = n - k - 1;
        double* v = sm + (size_t)(2 * cur) * n;
        double* w = v + n;
        double* vp = sm + (size_t)(2 * (cur ^ 1)) * n;
        const double* wp = vp + n;
        double* p = p2 + (size_t)(k & 1) * n;
        double* slot = slots + (size_t)(k & 1) * SYTRD_SLOTS;
        const bool pend = tprev != 0.0;
        // rows k+1 .. n-1: apply the pending update of step k-1 (cols >= k+1) and form
        // p = tau A22 v; the grid form also accumulates this warp's share of p.v
        double pvw = 0.0;
        for (int r = gwarp; r < m; r += nwarps) {
            double* arow = A + (size_t)(k + 1 + r) * lda + k + 1;
            const double vr = pend ? vp[r + 1] : 0.0, wr = pend ? wp[r + 1] : 0.0;
            // two FMAs per element for the rank-2 update, two accumulators for the dot (FP64
            // latency is long: independent chains keep the pipe busy)
            double s0 = 0.0, s1 = 0.0;
            double nx[RT];
            if (PREFETCH && r == gwarp && pre_ok) {
#pragma unroll
                for (int t = 0; t < RT; ++t) nx[t] = pre[t];
            } else {
#pragma unroll
                for (int t = 0; t < RT; ++t) {
                    const int c = lane + 32 * t;
                    nx[t] = c < m ? arow[c] : 0.0;
                }
            }
            for (int c0 = 0; c0 < m; c0 += 32 * RT) {
                double cu[RT];
#pragma unroll
                for (int t = 0; t < RT; ++t) cu[t] = nx[t];
#pragma unroll
                for (int t = 0; t < RT; ++t) {
                    const int c = c0 + 32 * RT + lane + 32 * t;
                    nx[t] = c < m ? arow[c] : 0.0;
                }
#pragma unroll
                for (int t = 0; t < RT; ++t) {
                    const int c = c0 + lane + 32 * t;
                    if (c < m) {
                        double a = cu[t];
                        if (pend) {
                            a = fma(-vr, wp[c + 1], a);
                            a = fma(-wr, vp[c + 1], a);
                            arow[c] = a;
                        }
                        if (t & 1) s1 = fma(a, v[c], s1);
                        else s0 = fma(a, v[c], s0);
                    }
                }
            }
            const double sdot = warp_sum(s0 + s1);
            const double pr = tk * sdot;
            if (lane == 0) p[r] = pr;
            if constexpr (!CTA) pvw = fma(pr, v[r], pvw);
        }
        if constexpr (CTA) {
            __syncthreads();
        } else {
            // this block's share of p.v: one value per warp, summed in warp order
            if (lane == 0) wred[wid] = pvw;
            __syncthreads();
            if (threadIdx.x == 0) slot[blockIdx.x] = sum_slots4(wred, (int)(blockDim.x >> 5));
            cg::this_grid().sync();
        }
        // p (for w = p - (tau/2)(p.v) v) and the next pivot row (row k+1, cols k+2..) are
        // loaded together: the pending buffers are free now, and the two loads share one trip
        // to L2
        const bool next = k + 1 < n - 2;
        pre_ok = PREFETCH && next && gwarp < m - 1;
        if (PREFETCH && pre_ok) {
            const double* arow = A + (size_t)(k + 2 + gwarp) * lda + k + 2;
#pragma unroll
            for (int t = 0; t < RT; ++t) {
                const int c = lane + 32 * t;
                pre[t] = c < m - 1 ? arow[c] : 0.0;
            }
        }
        double* xn = vp;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            if (tk != 0.0) w[i] = p[i];
            if (next && i < m - 1) xn[i] = A[(size_t)(k + 1) * lda + k + 2 + i];
        }
        if (tk != 0.0) {
            double pv;
            if constexpr (CTA) {
                pv = 0.0;
                for (int i = threadIdx.x; i < m; i += blockDim.x) pv += w[i] * v[i];
                pv = block_sum4(pv, red);
            } else {
                double t = 0.0;
                for (int b = lane; b < (int)gridDim.x; b += 32) t += slot[b];
                pv = warp_sum(t);
            }
            const double kk = -0.5 * tk * pv;
            for (int i = threadIdx.x; i < m; i += blockDim.x) w[i] += kk * v[i];
        }
        __syncthreads();
        tprev = tk;
        if (next) tk = reflector(k + 1, xn, v, w, tprev);
        cur ^= 1;
    }
    if (lead && threadIdx.x == 0) {
        if (n >= 3) {
            // rows n-2 and n-1 still carry the pending update of step n-3 (offset n-2)
            const double* vp = sm + (size_t)(2 * (cur ^ 1)) * n;
            const double* wp = vp + n;
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

// Number of eigenvalues of T below x, from the sign changes of the leading principal minors
// p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2}, p_{-1} = 1 (Sturm sequence, three-term form).
// Only one FMA per row sits on the dependent chain: d_i - x and e_{i-1}^2 p_{i-2} are formed
// off the chain, four rows at a time, and no division is needed (an FP64 divide costs about
// nine dependent FP64 operations on this part).  The pair (p_{i-1}, p_i) is rescaled by an
// exact power of two every four rows when its larger exponent leaves [2^-300, 2^300]; with
// e^2 floored at 2^-100 (d_tri_prep) four rows cannot move it out of the normal range, and
// no two consecutive minors can vanish, so a single zero minor gives exactly one sign change
// whichever sign it carries.  Sign and exponent tests use integer operations on the bits.
__device__ __forceinline__ int dexp_bits(double v) { return (__double2hiint(v) >> 20) & 0x7ff; }
__device__ __forceinline__ int sgn_change(double a, double b) { return (__double2hiint(a) ^ __double2hiint(b)) < 0; }

__device__ __forceinline__ void pair_rescale(double& pm, double& p) {
    const int ex = max(dexp_bits(p), dexp_bits(pm));
    if (ex > 1023 + 300) {
        p *= 0x1p-300;
        pm *= 0x1p-300;
    } else if (ex < 1023 - 300) {
        p *= 0x1p+300;
        pm *= 0x1p+300;
    }
}

__device__ inline int sturm_count(int n, const double* d, const double* e2, double x) {
    double pm = 1.0, p = d[0] - x;
    int cnt = __double2hiint(p) < 0;
    int i = 1;
    for (; i + 3 < n; i += 4) {
        const double t0 = d[i] - x, t1 = d[i + 1] - x, t2 = d[i + 2] - x, t3 = d[i + 3] - x;
        const double f0 = e2[i - 1], f1 = e2[i], f2 = e2[i + 1], f3 = e2[i + 2];
        const double p0 = fma(t0, p, -f0 * pm);
        const double p1 = fma(t1, p0, -f1 * p);
        const double p2 = fma(t2, p1, -f2 * p0);
        const double p3 = fma(t3, p2, -f3 * p1);
        cnt += sgn_change(p, p0) + sgn_change(p0, p1) + sgn_change(p1, p2) + sgn_change(p2, p3);
        pm = p2;
        p = p3;
        pair_rescale(pm, p);
    }
    for (; i < n; ++i) {
        const double pn = fma(d[i] - x, p, -e2[i - 1] * pm);
        cnt += sgn_change(p, pn);
        pm = p;
        p = pn;
        pair_rescale(pm, p);
    }
    return cnt;
}

// Newton correction -f(x)/f'(x) for f(x) = det(T - x I): the leading minors p_i and their
// derivatives p'_i follow p_i = (d_i - x) p_i-1 - e_i-1^2 p_i-2 and
// p'_i = (d_i - x) p'_i-1 - p_i-1 - e_i-1^2 p'_i-2.  The four running values are rescaled
// together by an exact power of two every four rows (the ratio is unchanged).
__device__ __forceinline__ void quad_rescale(double& pm, double& p, double& qm, double& q) {
    const int ex = max(max(dexp_bits(p), dexp_bits(pm)), max(dexp_bits(q), dexp_bits(qm)));
    if (ex > 1023 + 300) {
        p *= 0x1p-300; pm *= 0x1p-300; q *= 0x1p-300; qm *= 0x1p-300;
    } else if (ex < 1023 - 300) {
        p *= 0x1p+300; pm *= 0x1p+300; q *= 0x1p+300; qm *= 0x1p+300;
    }
}

__device__ inline double newton_dx(int n, const double* d, const double* e2, double x) {
    double pm = 1.0, p = d[0] - x, qm = 0.0, q = -1.0;
    int i = 1;
    for (; i + 3 < n; i += 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const double t = d[i + u] - x, f = e2[i + u - 1];
            const double pn = fma(t, p, -f * pm);
            const double qn = fma(t, q, -fma(f, qm, p));
            pm = p; p = pn; qm = q; q = qn;
        }
        quad_rescale(pm, p, qm, q);
    }
    for (; i < n; ++i) {
        const double t = d[i] - x, f = e2[i - 1];
        const double pn = fma(t, p, -f * pm);
        const double qn = fma(t, q, -fma(f, qm, p));
        pm = p; p = pn; qm = q; q = qn;
        quad_rescale(pm, p, qm, q);
    }
    return -p / q;
}

// The same count in FP32 with the ratio form q_i = (d_i - x) - e_{i-1}^2 / q_{i-1} and the
// pivmin guard; used only to narrow brackets that FP64 counts then verify.
__device__ inline int sturm_count32(int n, const float* d, const float* e2, float x, float pivmin) {
    float q = d[0] - x;
    if (fabsf(q) < pivmin) q = -pivmin;
    int cnt = q < 0.0f;
    for (int i = 1; i < n; ++i) {
        q = (d[i] - x) - __fdividef(e2[i - 1], q);
        if (fabsf(q) < pivmin) q = -pivmin;
        cnt += q < 0.0f;
    }
    return cnt;
}

__device__ inline void d_tri_prep(int n, const double* __restrict__ d, const double* __restrict__ e, double* __restrict__ e2,
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
            e2[i] = fmax(e[i] * e[i], 0x1p-100);   // floor: see sturm_count
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

// Eigenvalue j of T to an absolute accuracy of 2 eps ||T|| (the accuracy inverse iteration
// needs) by multisection: the G lanes of a group evaluate Sturm counts at G interior points of
// the bracket, which shrinks (G + 1)-fold per round.  The bracket is first
// narrowed with FP32 counts to about 1e-6 ||T||, widened by a margin far above the FP32
// backward error, and verified with two FP64 counts (falling back to the Gershgorin bracket
// if the check fails); FP64 rounds then finish it.  Must be called by all 32 lanes of a warp
// (lanes of inactive groups pass valid = false); d, e2 (FP64) and fd, fe2 (FP32 copies) are
// staged in shared memory.  Returns the eigenvalue in every lane of the group.
constexpr int BIS_G = 4;

// NEWTON: the FP64 phase starts with Newton steps (below).  It cuts the FP64 work about
// eightfold where the eigenvalues are well separated, which pays where FP64 throughput is the
// limit (the batched engine: +9% single points/s on the mixed set); on the plain engine's
// large clusters (many near-degenerate levels) Newton often falls back to multisection, and the
// latency-bound launch measured slower, so it is off there.
template <bool NEWTON, int G = BIS_G>
__device__ inline double d_bisect_group(int n, const double* sd, const double* se2, const float* fd, const float* fe2,
                                        const double* __restrict__ bounds, int j, bool valid) {
    const unsigned FULL = 0xffffffffu;
    static_assert(G >= 2 && G <= 32 && (G & (G - 1)) == 0, "group of 2..32 lanes, a power of two");
    const int lane = threadIdx.x & 31, gl = lane % G, gbase = lane - gl;
    const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << gbase;
    const double glo = bounds[0], ghi = bounds[1];
    const double tn = fmax(bounds[3], 1e-300);
    const double atol = 2.0 * 2.220446049250313e-16 * tn;
    // FP32 rounds
    const float ftol = (float)(1.0e-6 * tn);
    const float pivf = 1.0e-30f;
    float flo = (float)glo, fhi = (float)ghi;
    bool fact = valid;
    for (int r = 0; r < 48; ++r) {
        fact = fact && (fhi - flo > ftol);
        if (!__any_sync(FULL, fact)) break;
        const float h = (fhi - flo) / (float)(G + 1);
        const float x = flo + h * (float)(gl + 1);
        const int c = fact ? sturm_count32(n, fd, fe2, x, pivf) : 0;
        const unsigned bits = (__ballot_sync(FULL, fact && c > j) & gmask) >> gbase;
        if (fact) {
            const int k = bits ? __ffs(bits) - 1 : G;
            const float nlo = (k == 0) ? flo : flo + h * (float)k;
            const float nhi = (k == G) ? fhi : flo + h * (float)(k + 1);
            if (nlo == flo && nhi == fhi) fact = false;
            flo = nlo;
            fhi = nhi;
        }
    }
    // widen, verify with FP64 counts
    const double mar = 64.0 * 1.1920929e-7 * tn;
    double lo = fmax(glo, (double)flo - mar), hi = fmin(ghi, (double)fhi + mar);
    {
        const double xv = (gl == 0) ? lo : hi;
        const int c = (valid && gl < 2) ? sturm_count(n, sd, se2, xv) : 0;
        const unsigned okb = __ballot_sync(FULL, valid && ((gl == 0 && c <= j) || (gl == 1 && c > j)));
        const unsigned need = (3u << gbase);
        if (valid && (okb & need) != need) {
            lo = glo;
            hi = ghi;
        }
    }
    // FP64: Newton steps from the bracket's midpoint (lane 0 of the group), then two Sturm counts
    // confirm that eigenvalue j lies within eps*||T|| of x.  Quadratic convergence from the FP32
    // bracket takes about three steps; a cluster inside the bracket or a step that leaves it
    // falls back to multisection on the bracket.
    const double delta = 0.5 * atol;
    double x = 0.5 * (lo + hi);
    bool nwt = NEWTON && valid, nfail = !NEWTON;
    for (int it = 0; it < 6; ++it) {
        if (!__any_sync(FULL, nwt)) break;
        double dx = 0.0;
        if (nwt && gl == 0) dx = newton_dx(n, sd, se2, x);
        dx = __shfl_sync(FULL, dx, gbase);
        if (nwt) {
            const double xn = x + dx;
            if (!(xn > lo && xn < hi)) {
                nwt = false;
                nfail = true;
            } else {
                x = xn;
                if (fabs(dx) <= 0.25 * delta) nwt = false;
            }
        }
    }
    if (nwt) nfail = true;   // not converged within the step limit
    bool confirmed = false;
    {
        const bool chk = valid && !nfail && gl < 2;
        const int c = chk ? sturm_count(n, sd, se2, gl == 0 ? x - delta : x + delta) : 0;
        const unsigned okb = __ballot_sync(FULL, chk && ((gl == 0 && c <= j) || (gl == 1 && c > j)));
        const unsigned need = (3u << gbase);
        confirmed = valid && !nfail && (okb & need) == need;
        if (confirmed) {
            lo = x - delta;
            hi = x + delta;
        }
    }
    // FP64 multisection (only where Newton was not confirmed)
    bool act = valid && !confirmed;
    for (int r = 0; r < 80; ++r) {
        act = act && (hi - lo > atol);
        if (!__any_sync(FULL, act)) break;
        const double h = (hi - lo) / (double)(G + 1);
        const double x = lo + h * (double)(gl + 1);
        const int c = act ? sturm_count(n, sd, se2, x) : 0;
        const unsigned bits = (__ballot_sync(FULL, act && c > j) & gmask) >> gbase;
        if (act) {
            const int k = bits ? __ffs(bits) - 1 : G;
            const double nlo = (k == 0) ? lo : lo + h * (double)k;
            const double nhi = (k == G) ? hi : lo + h * (double)(k + 1);
            if (nlo == lo && nhi == hi) act = false;
            lo = nlo;
            hi = nhi;
        }
    }
    return 0.5 * (lo + hi);
}

// Stage d, e^2 and their FP32 copies (2n doubles followed by 2n floats) in shared memory.
__device__ inline void stage_tridiag(int n, const double* __restrict__ d, const double* __restrict__ e2, double* sm) {
    float* fsm = reinterpret_cast<float*>(sm + 2 * n);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double di = d[i], ei = (i < n - 1) ? e2[i] : 0.0;
        sm[i] = di;
        sm[n + i] = ei;
        fsm[i] = (float)di;
        fsm[n + i] = (float)ei;
    }
}

// |a| < |b| for doubles that are not NaN, by comparing the magnitude bits as integers.
__device__ __forceinline__ bool abs_less(double a, double b) {
    const unsigned long long m = 0x7fffffffffffffffULL;
    return ((unsigned long long)__double_as_longlong(a) & m) < ((unsigned long long)__double_as_longlong(b) & m);
}

// LU factors of T - lam I with partial pivoting, row i of U scaled by its pivot:
// U1 = 1/u_ii, U2 = u_i,i+1/u_ii, U3 = u_i,i+2/u_ii, ML = multiplier, piv = rows i, i+1
// interchanged.  The solve of (T - lam I) x = b is then
//   forward:  b_i <-> b_i+1 if piv_i; b_i+1 -= ML_i b_i
//   backward: x_i = U1_i b_i - U2_i x_i+1 - U3_i x_i+2
// so that one FMA per row sits on the dependent chain of the back substitution.

// Forward elimination of column j of Y in place, with the right-hand side scaled by `scale`
// as it is read (or, with gen != nullptr, generated on the fly).  Returns the last element,
// which is not stored.  Loads run CH rows ahead of the dependent chain.
template <int CH>
__device__ __forceinline__ double lu_forward(int n, double* __restrict__ y, size_t sn, const double* __restrict__ ml,
                                             const unsigned char* __restrict__ pv, double scale, uint32_t* gen) {
    auto rhs = [&](int i, double loaded) -> double {
        if (gen) {
            uint32_t s = *gen;
            s ^= s << 13; s ^= s >> 17; s ^= s << 5;
            *gen = s;
            return 0.5 + (double)(s & 0xffffff) / (double)0x1000000;
        }
        return loaded * scale;
    };
    double cur = rhs(0, gen ? 0.0 : y[0]);
    double nb[CH], nm[CH];
    unsigned char np[CH];
#pragma unroll
    for (int t = 0; t < CH; ++t) {
        const int i = t;
        const bool ok = i < n - 1;
        nb[t] = (ok && !gen) ? y[(size_t)(i + 1) * sn] : 0.0;
        nm[t] = ok ? ml[(size_t)i * sn] : 0.0;
        np[t] = ok ? pv[(size_t)i * sn] : 0;
    }
    for (int i0 = 0; i0 < n - 1; i0 += CH) {
        double cb[CH], cm[CH];
        unsigned char cp[CH];
#pragma unroll
        for (int t = 0; t < CH; ++t) { cb[t] = nb[t]; cm[t] = nm[t]; cp[t] = np[t]; }
#pragma unroll
        for (int t = 0; t < CH; ++t) {
            const int i = i0 + CH + t;
            const bool ok = i < n - 1;
            nb[t] = (ok && !gen) ? y[(size_t)(i + 1) * sn] : 0.0;
            nm[t] = ok ? ml[(size_t)i * sn] : 0.0;
            np[t] = ok ? pv[(size_t)i * sn] : 0;
        }
#pragma unroll
        for (int t = 0; t < CH; ++t) {
            const int i = i0 + t;
            if (i < n - 1) {
                const double bn = rhs(i + 1, cb[t]);
                const double bi = cp[t] ? bn : cur;
                const double bo = cp[t] ? cur : bn;
                y[(size_t)i * sn] = bi;
                cur = fma(-cm[t], bi, bo);
            }
        }
    }
    return cur;
}

// Back substitution of column j of Y in place; `last` is the forward result of row n-1.
// Returns max |x_i| and accumulates sum x_i^2 into *nrm2.
template <int CH>
__device__ __forceinline__ double lu_backward(int n, double* __restrict__ y, size_t sn, const double* __restrict__ u1,
                                              const double* __restrict__ u2, const double* __restrict__ u3,
                                              double last, double* nrm2) {
    double x1 = last * u1[(size_t)(n - 1) * sn], x2 = 0.0;
    y[(size_t)(n - 1) * sn] = x1;
    double mx = fabs(x1), s2 = x1 * x1;
    double nb[CH], n1[CH], n2[CH], n3[CH];
#pragma unroll
    for (int t = 0; t < CH; ++t) {
        const int i = n - 2 - t;
        const bool ok = i >= 0;
        const size_t o = ok ? (size_t)i * sn : 0;
        nb[t] = ok ? y[o] : 0.0;
        n1[t] = ok ? u1[o] : 0.0;
        n2[t] = ok ? u2[o] : 0.0;
        n3[t] = ok ? u3[o] : 0.0;
    }
    for (int i0 = n - 2; i0 >= 0; i0 -= CH) {
        double cb[CH], c1[CH], c2[CH], c3[CH];
#pragma unroll
        for (int t = 0; t < CH; ++t) { cb[t] = nb[t]; c1[t] = n1[t]; c2[t] = n2[t]; c3[t] = n3[t]; }
#pragma unroll
        for (int t = 0; t < CH; ++t) {
            const int i = i0 - CH - t;
            const bool ok = i >= 0;
            const size_t o = ok ? (size_t)i * sn : 0;
            nb[t] = ok ? y[o] : 0.0;
            n1[t] = ok ? u1[o] : 0.0;
            n2[t] = ok ? u2[o] : 0.0;
            n3[t] = ok ? u3[o] : 0.0;
        }
#pragma unroll
        for (int t = 0; t < CH; ++t) {
            const int i = i0 - t;
            if (i >= 0) {
                const double x = fma(-c2[t], x1, fma(-c3[t], x2, cb[t] * c1[t]));
                y[(size_t)i * sn] = x;
                x2 = x1;
                x1 = x;
                mx = fmax(mx, fabs(x));
                s2 = fma(x, x, s2);
            }
        }
    }
    *nrm2 = s2;
    return mx;
}

// Eigenvector j of T for eigenvalue w[j]; output Y[i*n + j].  Scratch arrays are
// [i*n + j] so that the threads of a warp (consecutive j) access consecutive words.
// Three steps of inverse iteration from a deterministic pseudo-random start (dstein's
// scheme without its convergence test); each step's right-hand side is the previous
// solution scaled by its largest element, and the result is normalised to unit length.
template <int CH = 8>
__device__ inline void d_inviter(int n, const double* __restrict__ d, const double* __restrict__ e,
                                 const double* __restrict__ w, const double* __restrict__ bounds, double* __restrict__ Y,
                                 double* __restrict__ U1, double* __restrict__ U2, double* __restrict__ U3,
                                 double* __restrict__ ML, unsigned char* __restrict__ piv, int j) {
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
    const size_t sn = (size_t)n;
    if (n == 1) { Y[j] = 1.0; return; }
    double* y = Y + j;
    double* u1 = U1 + j;
    double* u2 = U2 + j;
    double* u3 = U3 + j;
    double* ml = ML + j;
    unsigned char* pv = piv + j;
    // LU with partial pivoting of T - lam I.  Rows i (current: w0, w1, 0) and i+1
    // (e_i, d_i+1 - lam, e_i+1): the larger first entry becomes the pivot row.
    double w0 = d[0] - lam, w1 = e[0];
    for (int i = 0; i < n - 1; ++i) {
        const double sub = e[i];
        const double nd = d[i + 1] - lam;
        const double ns = (i + 1 < n - 1) ? e[i + 1] : 0.0;
        const bool sw = abs_less(w0, sub);
        double u0 = w0;
        if (!sw && abs_less(u0, pert)) u0 = copysign(pert, u0 == 0.0 ? 1.0 : u0);
        const double p0 = sw ? sub : u0, p1 = sw ? nd : w1, p2 = sw ? ns : 0.0;   // pivot row
        const double o0 = sw ? w0 : sub, o1 = sw ? w1 : nd, o2 = sw ? 0.0 : ns;   // eliminated row
        const double r0 = rcp_fast(p0);
        const double m = o0 * r0;
        const size_t o = (size_t)i * sn;
        u1[o] = r0;
        u2[o] = p1 * r0;
        u3[o] = p2 * r0;
        ml[o] = m;
        pv[o] = sw ? 1 : 0;
        w0 = fma(-o0 * p1, r0, o1);
        w1 = fma(-m, p2, o2);
    }
    if (abs_less(w0, pert)) w0 = copysign(pert, w0 == 0.0 ? 1.0 : w0);
    u1[(size_t)(n - 1) * sn] = rcp_fast(w0);
    uint32_t seed = 0x9e3779b9u ^ (uint32_t)(j * 2654435761u);
    double scale = 1.0, nrm2 = 1.0;
    for (int iter = 0; iter < 3; ++iter) {
        const double last = lu_forward<CH>(n, y, sn, ml, pv, scale, iter == 0 ? &seed : nullptr);
        const double mx = lu_backward<CH>(n, y, sn, u1, u2, u3, last, &nrm2);
        scale = 1.0 / mx;
    }
    const double sc = 1.0 / sqrt(nrm2);
    for (int i = 0; i < n; ++i) y[(size_t)i * sn] *= sc;
}

// One solve of (T - lam I) x = b for column j of Y with the factors of d_inviter (used by the
// cluster re-orthogonalisation).
__device__ inline void tri_solve_col(int n, int j, const double* __restrict__ U1, const double* __restrict__ U2,
                                     const double* __restrict__ U3, const double* __restrict__ ML,
                                     const unsigned char* __restrict__ piv, double* __restrict__ Y) {
    double nrm2;
    const double last = lu_forward<2>(n, Y + j, (size_t)n, ML + j, piv + j, 1.0, nullptr);
    lu_backward<2>(n, Y + j, (size_t)n, U1 + j, U2 + j, U3 + j, last, &nrm2);
}

// Clusters of (near-)degenerate eigenvalues (gap < ctol*||T||): inverse iteration with
// modified Gram-Schmidt against the earlier members after every solve (as dstein does).
// One warp per cluster, started by its first member; members are processed in order.
__device__ inline void d_reorth(int n, const double* __restrict__ w, const double* __restrict__ bounds, double ctol,
                         double* __restrict__ Y, const double* __restrict__ U1, const double* __restrict__ U2,
                         const double* __restrict__ U3, const double* __restrict__ ML,
                         const unsigned char* __restrict__ piv, int nc, int j, int lane) {
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


// ------------------------------------------------------------------ back-transformation
// Zt[j][:] = Q * Y[:, j] for every eigenvector j (one warp per eigenvector, vector staged in shared memory).
// y: n doubles of shared memory owned by the calling warp.
__device__ inline void d_ormtr_apply(int n, const double* __restrict__ V, const double* __restrict__ tau,
                                     const double* __restrict__ Y, int j, int lane, double* y) {
    for (int i = lane; i < n; i += 32) y[i] = Y[(size_t)i * n + j];
    __syncwarp();
    for (int k = n - 3; k >= 0; --k) {
        const double t = tau[k];
        if (t == 0.0) continue;
        const double* vk = V + (size_t)k * n;
        // four partial sums: with about one warp per scheduler nothing hides a single
        // 64-cycle dependent FMA chain
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int i = k + 1 + lane;
        for (; i + 96 < n; i += 128) {
            s0 = fma(vk[i], y[i], s0);
            s1 = fma(vk[i + 32], y[i + 32], s1);
            s2 = fma(vk[i + 64], y[i + 64], s2);
            s3 = fma(vk[i + 96], y[i + 96], s3);
        }
        for (; i < n; i += 32) s0 = fma(vk[i], y[i], s0);
        const double s = warp_sum((s0 + s1) + (s2 + s3)) * t;
        for (i = k + 1 + lane; i < n; i += 32) y[i] -= s * vk[i];
        __syncwarp();
    }
}

__device__ inline void d_ormtr(int n, const double* __restrict__ V, const double* __restrict__ tau,
                        const double* __restrict__ Y, double* __restrict__ Zt, int j, int lane, double* y) {
    d_ormtr_apply(n, V, tau, Y, j, lane, y);
    for (int i = lane; i < n; i += 32) Zt[(size_t)j * n + i] = y[i];
}

// Zt[j][:] = Q Y[:, j] for the columns j0 .. j0 + 31 below ncol, one column per lane of the
// calling warp, Y (row-major, updated in place) read and written a row of 32 columns at a time
// and each reflector broadcast from V.  A warp-wide FP64 instruction costs the same with one lane
// active as with 32, so this form spends about n^2 of them on 32 columns where the one-warp-per-
// column form spends n^2 / 32 + 7 n on each (its dot products end in a five-level shuffle sum).
// Lanes past ncol read column j0 (valid) and store nothing.
__device__ inline void d_ormtr_cols(int n, const double* __restrict__ V, const double* __restrict__ tau,
                                    double* __restrict__ Y, double* __restrict__ Zt, int j0, int ncol, int lane) {
    const int j = j0 + lane;
    const bool ok = j < ncol;
    double* yc = Y + (ok ? j : j0);
    for (int k = n - 3; k >= 0; --k) {
        const double t = tau[k];
        if (t == 0.0) continue;
        const double* vk = V + (size_t)k * n;
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int i = k + 1;
        for (; i + 3 < n; i += 4) {
            s0 = fma(vk[i], yc[(size_t)i * n], s0);
            s1 = fma(vk[i + 1], yc[(size_t)(i + 1) * n], s1);
            s2 = fma(vk[i + 2], yc[(size_t)(i + 2) * n], s2);
            s3 = fma(vk[i + 3], yc[(size_t)(i + 3) * n], s3);
        }
        for (; i < n; ++i) s0 = fma(vk[i], yc[(size_t)i * n], s0);
        const double s = ((s0 + s1) + (s2 + s3)) * t;
        if (ok)
            for (i = k + 1; i < n; ++i) yc[(size_t)i * n] = fma(-s, vk[i], yc[(size_t)i * n]);
    }
    if (ok)
        for (int i = 0; i < n; ++i) Zt[(size_t)j * n + i] = yc[(size_t)i * n];
}



// ------------------------------------------------------------------ one-block routines (batched engine)
// S = U^T U in place by one thread block (right-looking, unblocked; for the small matrices of
// the batched engine).  The strict lower triangle is zeroed.  Returns the first failing
// column + 1, or 0; the value is the same in every thread.
__device__ inline int cta_potrf_upper(int n, double* __restrict__ A, int lda) {
    __shared__ int bad;
    __shared__ double piv;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        if (threadIdx.x == 0) {
            double dkk = A[(size_t)k * lda + k];
            if (!(dkk > 0.0)) {
                if (bad == 0) bad = k + 1;
                dkk = 1.0;
            }
            piv = sqrt(dkk);
            A[(size_t)k * lda + k] = piv;
        }
        __syncthreads();
        const double dk = piv;
        for (int j = k + 1 + threadIdx.x; j < n; j += blockDim.x) A[(size_t)k * lda + j] /= dk;
        __syncthreads();
        const int m = n - k - 1;
        const double* uk = A + (size_t)k * lda;
        for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
            const int i = k + 1 + t / m, j = k + 1 + t % m;
            if (j >= i) A[(size_t)i * lda + j] -= uk[i] * uk[j];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int i = t / n, j = t % n;
        if (j < i) A[(size_t)i * lda + j] = 0.0;
    }
    __syncthreads();
    return bad;
}

// copy the lower triangle onto the upper one, one thread block
__device__ inline void cta_mirror_lower(int n, double* __restrict__ C, int ldc) {
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int i = t / n, j = t % n;
        if (j > i) C[(size_t)i * ldc + j] = C[(size_t)j * ldc + i];
    }
    __syncthreads();
}

}  // namespace xg
