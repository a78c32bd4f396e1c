// GFN2-xTB device kernels (FP64) for one molecule on sm_103a.
//
// Each kernel restates one piece of the reference single point; the reference
// routine is cited on the kernel.  Pair loops are written so that one warp or
// thread owns one output row (atom, shell or AO), which keeps every
// reduction deterministic; the only atomics are in the shell-pair gradient
// contraction and in the three-body dispersion gradient.
#include <cmath>

#include "gfn2_kernels.h"
#include "gfn2_device.cuh"

namespace xg {


__global__ void k_cn(DevMol m, int mode, double* __restrict__ cn) {
    const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (i >= m.nat) return;
    d_cn_warp(m, mode, cn, i, threadIdx.x & 31);
}


void cn(cudaStream_t st, const DevMol& m, int mode, double* out) {
    k_cn<<<ceil_div((long)m.nat * 32, 128), 128, 0, st>>>(m, mode, out);
    XG_LAUNCH_CHECK();
}


__global__ void k_cn_chain(DevMol m, int mode, const double* __restrict__ v, double* __restrict__ g) {
    const int a = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (a >= m.nat) return;
    d_cn_chain_warp(m, mode, v, g, a, threadIdx.x & 31);
}


void cn_chain(cudaStream_t st, const DevMol& m, int mode, const double* v, double* grad) {
    k_cn_chain<<<ceil_div((long)m.nat * 32, 128), 128, 0, st>>>(m, mode, v, grad);
    XG_LAUNCH_CHECK();
}


__global__ void k_eeq_matrix(DevMol m, const double* __restrict__ cn, double* __restrict__ A, double* __restrict__ X) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = m.nat;
    if (t >= (long)n * n) return;
    d_eeq_matrix(m, cn, A, X, t);
}


void eeq_setup(cudaStream_t st, const DevMol& m, const double* cnv, double* A, double* X) {
    k_eeq_matrix<<<ceil_div((long)m.nat * m.nat, 256), 256, 0, st>>>(m, cnv, A, X);
    XG_LAUNCH_CHECK();
}


__global__ void k_eeq_solve(int n, const double* __restrict__ U, double* __restrict__ X, double charge,
                            double* __restrict__ q) { d_eeq_solve(n, U, X, charge, q); }


// UT = U^T (n x n, 32 x 32 tiles through shared memory).
__global__ void k_transpose(int n, const double* __restrict__ U, double* __restrict__ UT) {
    __shared__ double tile[32][33];
    const int x = blockIdx.x * 32 + threadIdx.x;
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int y = blockIdx.y * 32 + yy;
        if (x < n && y < n) tile[yy][threadIdx.x] = U[(size_t)y * n + x];
    }
    __syncthreads();
    const int xo = blockIdx.y * 32 + threadIdx.x;
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int yo = blockIdx.x * 32 + yy;
        if (xo < n && yo < n) UT[(size_t)yo * n + xo] = tile[threadIdx.x][yy];
    }
}

// The two EEQ right-hand sides through U^T y = b and U x = y by one block, both as column
// sweeps (row i of U, then row i of U^T): one barrier per step and no reductions, with the
// right-hand sides and the reciprocal diagonal in shared memory (3 n doubles).  Then the
// charge constraint as in d_eeq_solve.
__global__ void __launch_bounds__(1024) k_eeq_solve_smem(int n, const double* __restrict__ U,
                                                         const double* __restrict__ UT, const double* __restrict__ X,
                                                         double charge, double* __restrict__ q) {
    extern __shared__ double es[];
    double* b0 = es;
    double* b1 = es + n;
    double* rd = es + 2 * n;
    __shared__ double red[32];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        b0[k] = X[k];
        b1[k] = X[n + k];
        rd[k] = 1.0 / U[(size_t)k * n + k];
    }
    __syncthreads();
    for (int i = 0; i < n; ++i) {
        const double y0 = b0[i] * rd[i], y1 = b1[i] * rd[i];
        const double* ur = U + (size_t)i * n;
        for (int k = i + 1 + threadIdx.x; k < n; k += blockDim.x) {
            const double u = ur[k];
            b0[k] = fma(-u, y0, b0[k]);
            b1[k] = fma(-u, y1, b1[k]);
        }
        __syncthreads();
        if (threadIdx.x == 0) { b0[i] = y0; b1[i] = y1; }
    }
    __syncthreads();
    for (int i = n - 1; i >= 0; --i) {
        const double x0 = b0[i] * rd[i], x1 = b1[i] * rd[i];
        const double* uc = UT + (size_t)i * n;   // column i of U
        for (int k = threadIdx.x; k < i; k += blockDim.x) {
            const double u = uc[k];
            b0[k] = fma(-u, x0, b0[k]);
            b1[k] = fma(-u, x1, b1[k]);
        }
        __syncthreads();
        if (threadIdx.x == 0) { b0[i] = x0; b1[i] = x1; }
    }
    __syncthreads();
    double sx0 = 0.0, sx1 = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) { sx0 += b0[k]; sx1 += b1[k]; }
    sx0 = block_sum(sx0, red);
    sx1 = block_sum(sx1, red);
    const double lam = (sx0 - charge) / sx1;
    for (int k = threadIdx.x; k < n; k += blockDim.x) q[k] = b0[k] - lam * b1[k];
}

void eeq_finish(cudaStream_t st, int nat, const double* Uf, double* X, double charge, double* q, double* work) {
    const size_t smem = 3 * (size_t)nat * sizeof(double);
    if (work && smem <= 200 * 1024) {
        k_transpose<<<dim3(ceil_div(nat, 32), ceil_div(nat, 32)), dim3(32, 8), 0, st>>>(nat, Uf, work);
        XG_LAUNCH_CHECK();
        if (smem > 48 * 1024) allow_max_dynamic_smem((const void*)k_eeq_solve_smem);
        k_eeq_solve_smem<<<1, 1024, smem, st>>>(nat, Uf, work, X, charge, q);
        XG_LAUNCH_CHECK();
        return;
    }
    k_eeq_solve<<<1, 1024, 0, st>>>(nat, Uf, X, charge, q);
    XG_LAUNCH_CHECK();
}


__global__ void k_dhdcn_diag(DevMol m, const double* __restrict__ P, double* __restrict__ dhdcn) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= m.nat) return;
    d_dhdcn_diag(m, P, dhdcn, a);
}


void dhdcn_diag(cudaStream_t st, const DevMol& m, const double* P, double* dhdcn) {
    k_dhdcn_diag<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, P, dhdcn);
    XG_LAUNCH_CHECK();
}


__global__ void k_jmat(DevMol m, double* __restrict__ J) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int ns = m.nsh;
    if (t >= (long)ns * ns) return;
    d_jmat(m, J, t);
}


void coulomb_matrix(cudaStream_t st, const DevMol& m, double* J) {
    k_jmat<<<ceil_div((long)m.nsh * m.nsh, 256), 256, 0, st>>>(m, J);
    XG_LAUNCH_CHECK();
}


__global__ void k_shell_shift(DevMol m, const double* __restrict__ J, const double* __restrict__ qsh,
                              const double* __restrict__ vat, double* __restrict__ shift, double* __restrict__ Jq) {
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (s >= m.nsh) return;
    d_shell_shift(m, J, qsh, vat, shift, Jq, s, lane);
}


void shell_shift(cudaStream_t st, const DevMol& m, const double* J, const double* qsh, const double* vat,
                 double* shift, double* Jq) {
    k_shell_shift<<<ceil_div((long)m.nsh * 32, 256), 256, 0, st>>>(m, J, qsh, vat, shift, Jq);
    XG_LAUNCH_CHECK();
}


__global__ void k_radcn(DevMol m, const double* __restrict__ cn, double* __restrict__ radcn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nat) return;
    d_radcn(m, cn, radcn, i);
}


__global__ void k_gab(DevMol m, const double* __restrict__ radcn, double* __restrict__ gab3, double* __restrict__ gab5) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = m.nat;
    if (t >= (long)n * n) return;
    d_gab(m, radcn, gab3, gab5, t);
}


void aes_setup(cudaStream_t st, const DevMol& m, const double* cnv, double* radcn, double* gab3, double* gab5) {
    k_radcn<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, cnv, radcn);
    XG_LAUNCH_CHECK();
    k_gab<<<ceil_div((long)m.nat * m.nat, 256), 256, 0, st>>>(m, radcn, gab3, gab5);
    XG_LAUNCH_CHECK();
}


__global__ void k_aes_pot(DevMol m, const double* __restrict__ q, const double* __restrict__ dipm,
                          const double* __restrict__ qp, const double* __restrict__ gab3, const double* __restrict__ gab5,
                          int shifted, double* __restrict__ vs, double* __restrict__ vd, double* __restrict__ vq) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= m.nat) return;
    d_aes_pot(m, q, dipm, qp, gab3, gab5, shifted, vs, vd, vq, i, lane);
}


void aes_potential(cudaStream_t st, const DevMol& m, const double* q, const double* dipm, const double* qp,
                   const double* gab3, const double* gab5, bool shifted, double* vs, double* vd, double* vq) {
    k_aes_pot<<<ceil_div((long)m.nat * 32, 128), 128, 0, st>>>(m, q, dipm, qp, gab3, gab5, shifted ? 1 : 0, vs, vd, vq);
    XG_LAUNCH_CHECK();
}


__global__ void k_aes_energy(DevMol m, const double* __restrict__ q, const double* __restrict__ dipm,
                             const double* __restrict__ qp, const double* __restrict__ gab3,
                             const double* __restrict__ gab5, double* __restrict__ e_part) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= m.nat) return;
    d_aes_energy(m, q, dipm, qp, gab3, gab5, e_part, i, lane);
}


void aes_energy(cudaStream_t st, const DevMol& m, const double* q, const double* dipm, const double* qp,
                const double* gab3, const double* gab5, double* e_part) {
    k_aes_energy<<<ceil_div((long)m.nat * 32, 128), 128, 0, st>>>(m, q, dipm, qp, gab3, gab5, e_part);
    XG_LAUNCH_CHECK();
}


__global__ void k_aes_grad(DevMol m, const double* __restrict__ q, const double* __restrict__ dipm,
                           const double* __restrict__ qp, const double* __restrict__ radcn,
                           const double* __restrict__ gab3, const double* __restrict__ gab5, double* __restrict__ grad,
                           double* __restrict__ tmp2) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= m.nat) return;
    d_aes_grad(m, q, dipm, qp, radcn, gab3, gab5, grad, tmp2, i, lane);
}


void aes_grad(cudaStream_t st, const DevMol& m, const double* q, const double* dipm, const double* qp,
              const double* radcn, const double* gab3, const double* gab5, double* grad, double* tmp2) {
    k_aes_grad<<<ceil_div((long)m.nat * 32, 128), 128, 0, st>>>(m, q, dipm, qp, radcn, gab3, gab5, grad, tmp2);
    XG_LAUNCH_CHECK();
}


__global__ void k_aes_dradcn(DevMol m, const double* __restrict__ cn, const double* __restrict__ tmp2,
                             double* __restrict__ dhdcn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nat) return;
    d_aes_dradcn(m, cn, tmp2, dhdcn, i);
}


void aes_dradcn(cudaStream_t st, const DevMol& m, const double* cnv, const double* tmp2, double* dhdcn) {
    k_aes_dradcn<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, cnv, tmp2, dhdcn);
    XG_LAUNCH_CHECK();
}


__global__ void k_build_h(DevMol m, double neglect, const double* __restrict__ H0, const double* __restrict__ S,
                          const double* __restrict__ D, const double* __restrict__ Q, const double* __restrict__ shift,
                          const double* __restrict__ vs, const double* __restrict__ vd, const double* __restrict__ vq,
                          double* __restrict__ H) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = m.nao;
    if (t >= (size_t)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    if (i > j) {
        H[t] = 0.0;
        return;
    }
    d_build_h(m, neglect, H0, S, D, Q, shift, vs, vd, vq, H, t);
    if (i == j) H[t] *= 0.5;
}


void build_hu(cudaStream_t st, const DevMol& m, Thresholds th, const double* H0, const double* S, const double* D,
              const double* Q, const double* shift, const double* vs, const double* vd, const double* vq, double* H) {
    const size_t nn = (size_t)m.nao * m.nao;
    k_build_h<<<ceil_div((long)nn, 256), 256, 0, st>>>(m, th.neglect, H0, S, D, Q, shift, vs, vd, vq, H);
    XG_LAUNCH_CHECK();
}


__global__ void k_fermi(int n, const double* __restrict__ emo, int nel_a, int nel_b, double etemp,
                        double* __restrict__ focc, double* __restrict__ fa, double* __restrict__ fb,
                        double* __restrict__ scal, int* __restrict__ kocc, const int* __restrict__ gate) {
    if (gate && *gate == 0) return;
    d_fermi(n, emo, nel_a, nel_b, etemp, focc, fa, fb, scal, kocc);
}


void fermi(cudaStream_t st, int n, const double* emo, int nel_a, int nel_b, double etemp, double* focc, double* fa,
           double* fb, double* scal, int* kocc, const int* gate) {
    k_fermi<<<1, 1024, 0, st>>>(n, emo, nel_a, nel_b, etemp, focc, fa, fb, scal, kocc, gate);
    XG_LAUNCH_CHECK();
}


__global__ void k_scale_cols(int n, const double* __restrict__ C, const double* __restrict__ f, double* __restrict__ Cf) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * n) return;
    d_scale_cols(n, C, f, Cf, t);
}


void scale_cols(cudaStream_t st, int n, const double* C, const double* f, double* Cf) {
    k_scale_cols<<<ceil_div((long)n * n, 256), 256, 0, st>>>(n, C, f, Cf);
    XG_LAUNCH_CHECK();
}


__global__ void k_rowsums(DevMol m, const double* __restrict__ P, const double* __restrict__ S,
                          const double* __restrict__ D, const double* __restrict__ Q, const double* __restrict__ H0,
                          double* __restrict__ rows) {
    const int mu = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (mu >= m.nao) return;
    d_rowsums(m, P, S, D, Q, H0, rows, mu, lane);
}


__global__ void k_atom_pop(DevMol m, const double* __restrict__ rows, double* __restrict__ qsh, double* __restrict__ q,
                           double* __restrict__ dipm, double* __restrict__ qp, double* __restrict__ eh0) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= m.nat) return;
    d_atom_pop(m, rows, qsh, q, dipm, qp, eh0, a);
}


void populations(cudaStream_t st, const DevMol& m, const double* P, const double* S, const double* D, const double* Q,
                 const double* H0, double* rows, double* qsh, double* q, double* dipm, double* qp, double* eh0) {
    k_rowsums<<<ceil_div((long)m.nao * 32, 256), 256, 0, st>>>(m, P, S, D, Q, H0, rows);
    XG_LAUNCH_CHECK();
    k_atom_pop<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, rows, qsh, q, dipm, qp, eh0);
    XG_LAUNCH_CHECK();
}


__global__ void k_reduce(const double* __restrict__ x, int n, double* __restrict__ out) { d_reduce(x, n, out); }


void reduce_sum(cudaStream_t st, const double* x, int n, double* out) {
    k_reduce<<<1, 512, 0, st>>>(x, n, out);
    XG_LAUNCH_CHECK();
}


__global__ void k_add(int n, const double* __restrict__ a, double* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] += a[i];
}

void add_vec(cudaStream_t st, int n, const double* a, double* b) {
    k_add<<<ceil_div(n, 256), 256, 0, st>>>(n, a, b);
    XG_LAUNCH_CHECK();
}


// ================================================================== Broyden mixing
// broyden (src/broyden.f90:37-153) with gfn2broyden_save/diff/out packing (src/aespot.F90:1360-1425)


__global__ void k_broyden_pack(DevMol m, const double* __restrict__ qsh, const double* __restrict__ dipm,
                               const double* __restrict__ qp, double* __restrict__ v) {
    d_broyden_pack(m, qsh, dipm, qp, v, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_broyden_unpack(DevMol m, const double* __restrict__ v, double* __restrict__ qsh,
                                 double* __restrict__ dipm, double* __restrict__ qp, double* __restrict__ q) {
    d_broyden_unpack(m, v, qsh, dipm, qp, q, blockIdx.x * blockDim.x + threadIdx.x);
}
void broyden_pack(cudaStream_t st, const DevMol& m, const double* qsh, const double* dipm, const double* qp, double* vec) {
    k_broyden_pack<<<ceil_div(std::max(m.nsh, m.nat), 256), 256, 0, st>>>(m, qsh, dipm, qp, vec);
    XG_LAUNCH_CHECK();
}

void broyden_unpack(cudaStream_t st, const DevMol& m, const double* vec, double* qsh, double* dipm, double* qp, double* q) {
    k_broyden_unpack<<<ceil_div(std::max(m.nsh, m.nat), 256), 256, 0, st>>>(m, vec, qsh, dipm, qp, q);
    XG_LAUNCH_CHECK();
}


__global__ void k_broyden(int nbr, int it, int maxit, double alpha, double* __restrict__ qin,
                          const double* __restrict__ qout, double* __restrict__ dq, double* __restrict__ df,
                          double* __restrict__ u, double* __restrict__ amat, double* __restrict__ omega,
                          double* __restrict__ qlast, double* __restrict__ dqlast, double* __restrict__ work,
                          double* __restrict__ rms_out, int nat) { d_broyden(nbr, it, maxit, alpha, qin, qout, dq, df, u, amat, omega, qlast, dqlast, work, rms_out, nat); }


void broyden_step(cudaStream_t st, BroydenState& bs, int it, double alpha, double* qin, const double* qout, double* dq,
                  double* rms_out, int nat) {
    k_broyden<<<1, 1024, 0, st>>>(bs.nbr, it, bs.maxit, alpha, qin, qout, dq, bs.df, bs.u, bs.a, bs.omega, bs.qlast,
                                  bs.dqlast, bs.scratch, rms_out, nat);
    XG_LAUNCH_CHECK();
}


__global__ void k_repulsion(DevMol m, double* __restrict__ e_atom, double* __restrict__ grad) {
    const int a = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (a >= m.nat) return;
    d_repulsion_warp(m, e_atom, grad, a, threadIdx.x & 31);
}


void repulsion(cudaStream_t st, const DevMol& m, double* e_atom, double* grad) {
    k_repulsion<<<ceil_div((long)m.nat * 32, 128), 128, 0, st>>>(m, e_atom, grad);
    XG_LAUNCH_CHECK();
}


__global__ void k_coulomb_grad(DevMol m, const double* __restrict__ qsh, double* __restrict__ grad) {
    const int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (a >= m.nat) return;
    d_coulomb_grad(m, qsh, grad, a, lane);
}


void coulomb_grad(cudaStream_t st, const DevMol& m, const double* qsh, double* grad) {
    k_coulomb_grad<<<ceil_div((long)m.nat * 32, 128), 128, 0, st>>>(m, qsh, grad);
    XG_LAUNCH_CHECK();
}


__global__ void k_d4_weights(DevMol m, const double* __restrict__ cnv, double* __restrict__ gw, double* __restrict__ dgw) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= m.nat) return;
    d_d4_weights(m, cnv, gw, dgw, a);
}


void d4_weights(cudaStream_t st, const DevMol& m, const double* cnv, double* gw, double* dgw) {
    k_d4_weights<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, cnv, gw, dgw);
    XG_LAUNCH_CHECK();
}


__global__ void k_d4_zeta(DevMol m, const double* __restrict__ gw, const double* __restrict__ q,
                          double* __restrict__ zeta, double* __restrict__ dzeta) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= m.nat) return;
    d_d4_zeta(m, gw, q, zeta, dzeta, a);
}


__global__ void k_d4_wz(DevMol m, const double* __restrict__ gw, const double* __restrict__ zeta,
                        const double* __restrict__ dzeta, double* __restrict__ Wz, double* __restrict__ vat,
                        double* __restrict__ e_atom) {
    const int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (a >= m.nat) return;
    d_d4_wz(m, gw, zeta, dzeta, Wz, vat, e_atom, a, lane);
}


void d4_scc(cudaStream_t st, const DevMol& m, const double* gw, const double* q, double* zeta, double* dzeta,
            double* Wz, double* vat, double* e_atom) {
    k_d4_zeta<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, gw, q, zeta, dzeta);
    XG_LAUNCH_CHECK();
    k_d4_wz<<<ceil_div((long)m.nat * 32, 128), 128, 0, st>>>(m, gw, zeta, dzeta, Wz, vat, e_atom);
    XG_LAUNCH_CHECK();
}


__global__ void k_d4_refvec(DevMol m, const double* __restrict__ gw, const double* __restrict__ dgw,
                            const double* __restrict__ q, double* __restrict__ zv, double* __restrict__ zr,
                            double* __restrict__ zdcn, double* __restrict__ zrdcn) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= m.nat) return;
    d_d4_refvec(m, gw, dgw, q, zv, zr, zdcn, zrdcn, a);
}


__global__ void k_d4_c6(DevMol m, const double* __restrict__ zv, const double* __restrict__ zdcn,
                        double* __restrict__ c6o, double* __restrict__ dc6o) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = m.nat;
    if (t >= (long)n * n) return;
    d_d4_c6(m, zv, zdcn, c6o, dc6o, t);
}


__global__ void k_d4_2body(DevMol m, const double* __restrict__ c6, const double* __restrict__ dc6,
                           double* __restrict__ e_atom, double* __restrict__ dEdcn, double* __restrict__ grad) {
    const int a = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (a >= m.nat) return;
    d_d4_2body_warp(m, c6, dc6, e_atom, dEdcn, grad, a, threadIdx.x & 31);
}


// ATM three-body (atm_gradient_latp molecular branch + deriv_atm_triple, src/disp/dftd4.F90:2023-2177, 2354-2433).
// The triple terms factor into pair quantities: the damping base (C_ijk / R_ijk)^(16/3) with
// C_ijk = c_ij c_ik c_jk and R_ijk = R_ij R_ik R_jk is tp_ij tp_ik tp_jk, tp = (c / R)^(16/3);
// sqrt(C6_ij C6_ik C6_jk) is s6_ij s6_ik s6_jk; 1/R_ijk is ir_ij ir_ik ir_jk.  k_atm_pairs
// forms them once per pair (t = a*n + b), so the O(N^3) loop has no power, square root or
// division other than the damping's reciprocal.  ga[a*n + b] = (dC6_ab/dCN_a) / C6_ab and its
// transpose gt serve the C6 derivatives with coalesced loads for either index order.
__global__ void k_atm_pairs(DevMol m, const double* __restrict__ c6, const double* __restrict__ dc6,
                            double* __restrict__ ir, double* __restrict__ tp, double* __restrict__ s6,
                            double* __restrict__ ga, double* __restrict__ gt) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = m.nat;
    if (t >= (long)n * n) return;
    const int a = (int)(t / n), b = (int)(t % n);
    const size_t tt = (size_t)b * n + a;
    if (a == b) {
        ir[t] = 0.0; tp[t] = 0.0; s6[t] = 0.0; ga[t] = 0.0; gt[t] = 0.0;
        return;
    }
    const double dx = m.xyz[3 * b] - m.xyz[3 * a], dy = m.xyz[3 * b + 1] - m.xyz[3 * a + 1],
                 dz = m.xyz[3 * b + 2] - m.xyz[3 * a + 2];
    const double irr = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
    const double cab = 0.52 * sqrt(3.0 * m.r4r2[a] * m.r4r2[b]) + 5.0;
    ir[t] = irr;
    tp[t] = pow(cab * irr, 16.0 / 3.0);
    s6[t] = sqrt(c6[t]);
    const double g = dc6[t] / c6[tt];
    ga[t] = g;
    gt[tt] = g;
}

// One thread per pair (i > j), loop over k < j; gradient and dE/dCN of k by atomics.  The terms
// of i and j that share a factor across k (the i-j distance vector, the C6 derivative ratios of
// the pair) are summed over k first and applied once after the loop.
__global__ void k_d4_atm(DevMol m, const double* __restrict__ ir, const double* __restrict__ tp,
                         const double* __restrict__ s6, const double* __restrict__ ga, const double* __restrict__ gt,
                         long npair, double* __restrict__ e_pair, double* __restrict__ dEdcn,
                         double* __restrict__ grad) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npair) return;
    int ia, ja;
    tri_pair(t, ia, ja);
    if (ja >= ia) { e_pair[t] = 0.0; return; }
    const int n = m.nat;
    const double cut2 = 1600.0, s9 = 5.0;
    const double* x = m.xyz;
    const double rij[3] = {x[3 * ja] - x[3 * ia], x[3 * ja + 1] - x[3 * ia + 1], x[3 * ja + 2] - x[3 * ia + 2]};
    const double r2ij = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
    double esum = 0.0;
    if (r2ij <= cut2) {
        // gi = -(S1 rij + sum_k dGr2 rik), gj = S1 rij - sum_k dGr3 rjk with S1 = sum_k dGr1;
        // dci = gi_j H + sum_k h gt_ik, dcj = gj_i H + sum_k h gt_jk with H = sum_k h
        double gik[3] = {0, 0, 0}, gjk[3] = {0, 0, 0}, s1 = 0.0, hs = 0.0, dci = 0.0, dcj = 0.0;
        const size_t pij = (size_t)ja * n + ia;
        const double irij = ir[pij], tij = tp[pij], sij = s6[pij];
        const double gi_j = ga[(size_t)ia * n + ja], gj_i = ga[pij];
        const double w1 = s9 * irij * irij;
        for (int ka = 0; ka < ja; ++ka) {
            const double rik[3] = {x[3 * ka] - x[3 * ia], x[3 * ka + 1] - x[3 * ia + 1], x[3 * ka + 2] - x[3 * ia + 2]};
            const double r2ik = rik[0] * rik[0] + rik[1] * rik[1] + rik[2] * rik[2];
            if (r2ik > cut2) continue;
            const double rjk[3] = {x[3 * ka] - x[3 * ja], x[3 * ka + 1] - x[3 * ja + 1], x[3 * ka + 2] - x[3 * ja + 2]};
            const double r2jk = rjk[0] * rjk[0] + rjk[1] * rjk[1] + rjk[2] * rjk[2];
            if (r2jk > cut2) continue;
            const size_t pik = (size_t)ka * n + ia, pjk = (size_t)ka * n + ja;
            const double irik = ir[pik], irjk = ir[pjk];
            const double c9 = -(sij * s6[pik] * s6[pjk]);
            const double cralp = tij * tp[pik] * tp[pjk];
            const double irrr1 = irij * irik * irjk;
            const double irrr2 = irrr1 * irrr1, irrr3 = irrr2 * irrr1;
            const double ang_fact = 0.375 * irrr2 * irrr3;
            const double ang = ang_fact * (r2ij + r2jk - r2ik) * (r2ij - r2jk + r2ik) * (-r2ij + r2jk + r2ik) + irrr3;
            const double fdmp = rcp_fast(1.0 + 6.0 * cralp);
            const double dfdmp = -(2.0 * 16.0 * cralp) * fdmp * fdmp;
            const double c9f = c9 * fdmp, c9d = dfdmp * c9 * ang;
            // dGr_x = s9 (c9d - dang_x c9f) / r_x^2 with dang_x = -ang_fact P_x
            const double qf = ang_fact * c9f;
            const double dGr1 = fma(qf, atm_dpoly(r2ij, r2jk, r2ik), c9d) * w1;
            const double dGr2 = fma(qf, atm_dpoly(r2ik, r2jk, r2ij), c9d) * (s9 * irik * irik);
            const double dGr3 = fma(qf, atm_dpoly(r2jk, r2ik, r2ij), c9d) * (s9 * irjk * irjk);
            esum = fma(-ang, c9f, esum);
            s1 += dGr1;
            for (int q = 0; q < 3; ++q) {
                const double a2 = dGr2 * rik[q], a3 = dGr3 * rjk[q];
                gik[q] += a2;
                gjk[q] += a3;
                atomicAdd(&grad[3 * ka + q], a2 + a3);
            }
            const double h = (-0.5 * s9) * ang * c9f;
            hs += h;
            dci = fma(h, gt[pik], dci);
            dcj = fma(h, gt[pjk], dcj);
            atomicAdd(&dEdcn[ka], h * (ga[pik] + ga[pjk]));
        }
        for (int q = 0; q < 3; ++q) {
            atomicAdd(&grad[3 * ia + q], -fma(s1, rij[q], gik[q]));
            atomicAdd(&grad[3 * ja + q], fma(s1, rij[q], -gjk[q]));
        }
        atomicAdd(&dEdcn[ia], fma(gi_j, hs, dci));
        atomicAdd(&dEdcn[ja], fma(gj_i, hs, dcj));
        esum *= s9;
    }
    e_pair[t] = esum;
}

void d4_grad(cudaStream_t st, const DevMol& m, const double* cnv, const double* q, double* gw, double* dgw,
             double* zv, double* zr, double* zdcn, double* zrdcn, double* c6, double* dc6, double* c6z, double* dc6z,
             double* e2_atom, double* e3_pair, double* dEdcn, double* grad, double* pair_work) {
    k_d4_weights<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, cnv, gw, dgw);
    XG_LAUNCH_CHECK();
    k_d4_refvec<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, gw, dgw, q, zv, zr, zdcn, zrdcn);
    XG_LAUNCH_CHECK();
    const long nn = (long)m.nat * m.nat;
    k_d4_c6<<<ceil_div(nn, 256), 256, 0, st>>>(m, zv, zdcn, c6, dc6);
    XG_LAUNCH_CHECK();
    k_d4_c6<<<ceil_div(nn, 256), 256, 0, st>>>(m, zr, zrdcn, c6z, dc6z);
    XG_LAUNCH_CHECK();
    k_d4_2body<<<ceil_div((long)m.nat * 32, 128), 128, 0, st>>>(m, c6, dc6, e2_atom, dEdcn, grad);
    XG_LAUNCH_CHECK();
    // ATM pair factors: c6 and dc6 are free once the two-body term is done
    double* ir = c6;
    double* tp = dc6;
    double* s6 = pair_work;
    double* ga = pair_work + nn;
    double* gt = pair_work + 2 * nn;
    k_atm_pairs<<<ceil_div(nn, 256), 256, 0, st>>>(m, c6z, dc6z, ir, tp, s6, ga, gt);
    XG_LAUNCH_CHECK();
    const long np = (long)m.nat * (m.nat + 1) / 2;
    k_d4_atm<<<ceil_div(np, 128), 128, 0, st>>>(m, ir, tp, s6, ga, gt, np, e3_pair, dEdcn, grad);
    XG_LAUNCH_CHECK();
}

}  // namespace xg
