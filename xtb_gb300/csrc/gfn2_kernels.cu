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
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nat) return;
    d_cn(m, mode, cn, i);
}


void cn(cudaStream_t st, const DevMol& m, int mode, double* out) {
    k_cn<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, mode, out);
    XG_LAUNCH_CHECK();
}


__global__ void k_cn_chain(DevMol m, int mode, const double* __restrict__ v, double* __restrict__ g) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= m.nat) return;
    d_cn_chain(m, mode, v, g, a);
}


void cn_chain(cudaStream_t st, const DevMol& m, int mode, const double* v, double* grad) {
    k_cn_chain<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, mode, v, grad);
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


void eeq_finish(cudaStream_t st, int nat, const double* Uf, double* X, double charge, double* q, double*) {
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
    if (t >= (size_t)m.nao * m.nao) return;
    d_build_h(m, neglect, H0, S, D, Q, shift, vs, vd, vq, H, t);
}


void build_h(cudaStream_t st, const DevMol& m, Thresholds th, const double* H0, const double* S, const double* D,
             const double* Q, const double* shift, const double* vs, const double* vd, const double* vq, double* H) {
    const size_t nn = (size_t)m.nao * m.nao;
    k_build_h<<<ceil_div((long)nn, 256), 256, 0, st>>>(m, th.neglect, H0, S, D, Q, shift, vs, vd, vq, H);
    XG_LAUNCH_CHECK();
}


__global__ void k_fermi(int n, const double* __restrict__ emo, int nel_a, int nel_b, double etemp,
                        double* __restrict__ focc, double* __restrict__ fa, double* __restrict__ fb,
                        double* __restrict__ scal, int* __restrict__ kocc) { d_fermi(n, emo, nel_a, nel_b, etemp, focc, fa, fb, scal, kocc); }


void fermi(cudaStream_t st, int n, const double* emo, int nel_a, int nel_b, double etemp, double* focc, double* fa,
           double* fb, double* scal, int* kocc) {
    k_fermi<<<1, 1024, 0, st>>>(n, emo, nel_a, nel_b, etemp, focc, fa, fb, scal, kocc);
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
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= m.nat) return;
    d_repulsion(m, e_atom, grad, a);
}


void repulsion(cudaStream_t st, const DevMol& m, double* e_atom, double* grad) {
    k_repulsion<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, e_atom, grad);
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
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= m.nat) return;
    d_d4_2body(m, c6, dc6, e_atom, dEdcn, grad, a);
}


// ATM three-body (atm_gradient_latp molecular branch + deriv_atm_triple, src/disp/dftd4.F90:2023-2177, 2354-2433);
// one thread per pair (i > j), loop over k < j; gradient and dE/dCN of j, k by atomics.


__global__ void k_d4_atm(DevMol m, const double* __restrict__ c6, const double* __restrict__ dc6, long npair,
                         double* __restrict__ e_pair, double* __restrict__ dEdcn, double* __restrict__ grad) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npair) return;
    d_d4_atm(m, c6, dc6, npair, e_pair, dEdcn, grad, t);
}
void d4_grad(cudaStream_t st, const DevMol& m, const double* cnv, const double* q, double* gw, double* dgw,
             double* zv, double* zr, double* zdcn, double* zrdcn, double* c6, double* dc6, double* c6z, double* dc6z,
             double* e2_atom, double* e3_pair, double* dEdcn, double* grad) {
    k_d4_weights<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, cnv, gw, dgw);
    XG_LAUNCH_CHECK();
    k_d4_refvec<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, gw, dgw, q, zv, zr, zdcn, zrdcn);
    XG_LAUNCH_CHECK();
    const long nn = (long)m.nat * m.nat;
    k_d4_c6<<<ceil_div(nn, 256), 256, 0, st>>>(m, zv, zdcn, c6, dc6);
    XG_LAUNCH_CHECK();
    k_d4_c6<<<ceil_div(nn, 256), 256, 0, st>>>(m, zr, zrdcn, c6z, dc6z);
    XG_LAUNCH_CHECK();
    k_d4_2body<<<ceil_div(m.nat, 128), 128, 0, st>>>(m, c6, dc6, e2_atom, dEdcn, grad);
    XG_LAUNCH_CHECK();
    const long np = (long)m.nat * (m.nat + 1) / 2;
    k_d4_atm<<<ceil_div(np, 128), 128, 0, st>>>(m, c6z, dc6z, np, e3_pair, dEdcn, grad);
    XG_LAUNCH_CHECK();
}

}  // namespace xg
