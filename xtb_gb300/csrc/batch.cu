// Batched GFN2-xTB single points: one thread block per molecule (sm_103a, FP64).
//
// The device program of one molecule restates the plain engine's sequence
// (scf, src/scf_module.F90:74-920; scc, src/scc_core.f90:255-640) with the same
// device bodies; the dense linear algebra (Cholesky, X^T H X, Householder
// tridiagonalisation, bisection, inverse iteration, back-transformation, density)
// runs inside the block.  Molecules keep their whole state in device memory
// between launches, so a launch can take every molecule to completion or advance
// it by a few SCC iterations only.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "batch.h"
#include "gfn2_device.cuh"
#include "linalg_device.cuh"

namespace xg {

namespace {

constexpr int BT = 256;   // threads per molecule block

// ------------------------------------------------------------------ layout
// Carves the arrays of one molecule out of the batch allocation (two passes:
// count with base == nullptr, then assign).  Parameter arrays are recorded with
// their host source so that they can be staged into one upload buffer.
struct Carver {
    char* base = nullptr;
    size_t used = 0;
    struct Up { size_t off; const void* src; size_t bytes; };
    std::vector<Up>* ups = nullptr;
    template <typename T>
    T* take(size_t count) {
        const size_t bytes = ((std::max<size_t>(count, 1) * sizeof(T) + 255) / 256) * 256;
        T* p = base ? reinterpret_cast<T*>(base + used) : nullptr;
        used += bytes;
        return p;
    }
    template <typename T>
    const T* upload(const std::vector<T>& v) {
        const size_t off = used;
        T* p = take<T>(v.size());
        if (ups && !v.empty()) ups->push_back({off, v.data(), v.size() * sizeof(T)});
        return p;
    }
};

void layout_mol(Carver& cv, const HostMol& hm, BatchMol& b, const std::vector<double>* guess = nullptr) {
    const int nat = hm.nat, nsh = hm.nsh, nao = hm.nao;
    const size_t nn = (size_t)nao * nao, aa = (size_t)nat * nat;
    DevMol& m = b.m;
    m.nat = nat; m.nsh = nsh; m.nao = nao; m.nelem = hm.nelem;
    m.Z = cv.upload(hm.Z); m.eid = cv.upload(hm.eid); m.xyz = cv.upload(hm.xyz);
    m.at_sh0 = cv.upload(hm.at_sh0); m.at_nsh = cv.upload(hm.at_nsh);
    m.at_ao0 = cv.upload(hm.at_ao0); m.at_nao = cv.upload(hm.at_nao);
    m.rcov = cv.upload(hm.rcov); m.en = cv.upload(hm.en); m.rcov4 = cv.upload(hm.rcov4); m.en4 = cv.upload(hm.en4);
    m.eeq_en = cv.upload(hm.eeq_en); m.eeq_gam = cv.upload(hm.eeq_gam);
    m.eeq_kappa = cv.upload(hm.eeq_kappa); m.eeq_alpha = cv.upload(hm.eeq_alpha);
    m.mrad = cv.upload(hm.mrad); m.valcn = cv.upload(hm.valcn); m.dkern = cv.upload(hm.dkern);
    m.qkern = cv.upload(hm.qkern); m.rep_alpha = cv.upload(hm.rep_alpha); m.rep_zeff = cv.upload(hm.rep_zeff);
    m.r4r2 = cv.upload(hm.r4r2); m.arad = cv.upload(hm.arad);
    m.d4_nref = cv.upload(hm.d4_nref); m.d4_zeff = cv.upload(hm.d4_zeff); m.d4_gam = cv.upload(hm.d4_gam);
    m.d4_refq = cv.upload(hm.d4_refq); m.d4_refcn = cv.upload(hm.d4_refcn);
    m.d4_ncount = cv.upload(hm.d4_ncount); m.d4_c6 = cv.upload(hm.d4_c6);
    m.sh_atom = cv.upload(hm.sh_atom); m.sh_l = cv.upload(hm.sh_l); m.sh_ao = cv.upload(hm.sh_ao);
    m.sh_nprim = cv.upload(hm.sh_nprim); m.sh_alpha = cv.upload(hm.sh_alpha); m.sh_coef = cv.upload(hm.sh_coef);
    m.sh_zeta = cv.upload(hm.sh_zeta); m.sh_se0 = cv.upload(hm.sh_se0); m.sh_kcn = cv.upload(hm.sh_kcn);
    m.sh_poly = cv.upload(hm.sh_poly); m.sh_eta = cv.upload(hm.sh_eta); m.sh_gam3 = cv.upload(hm.sh_gam3);
    m.sh_zsh = cv.upload(hm.sh_zsh);
    m.ao_sh = cv.upload(hm.ao_sh); m.ao_at = cv.upload(hm.ao_at);
    m.sh_byl = cv.upload(hm.sh_byl);
    for (int l = 0; l < 4; ++l) m.l_off[l] = hm.l_off[l];
    b.zval = cv.upload(hm.zval);
    b.guess = guess ? cv.upload(*guess) : nullptr;

    b.S = cv.take<double>(nn); b.D = cv.take<double>(3 * nn); b.Q = cv.take<double>(6 * nn);
    b.H0 = cv.take<double>(nn); b.X = cv.take<double>(nn); b.H = cv.take<double>(nn); b.A = cv.take<double>(nn);
    b.T1 = cv.take<double>(nn); b.C = cv.take<double>(nn); b.P = cv.take<double>(nn); b.W = cv.take<double>(nn);
    b.V = cv.take<double>(nn); b.Y = cv.take<double>(nn); b.Zt = cv.take<double>(nn);
    b.iscr = cv.take<double>(4 * nn); b.piv = cv.take<unsigned char>(nn);
    b.J = cv.take<double>((size_t)nsh * nsh);
    b.gab3 = cv.take<double>(aa); b.gab5 = cv.take<double>(aa); b.c6 = cv.take<double>(aa);
    b.dc6 = cv.take<double>(aa); b.c6z = cv.take<double>(aa); b.dc6z = cv.take<double>(aa);
    b.eeqA = cv.take<double>(aa); b.eeqX = cv.take<double>(2 * (size_t)nat);
    b.cn_gfn = cv.take<double>(nat); b.cn_tmp = cv.take<double>(nat); b.se = cv.take<double>(nsh);
    b.q = cv.take<double>(nat); b.qsh = cv.take<double>(nsh); b.dipm = cv.take<double>(3 * (size_t)nat);
    b.qp = cv.take<double>(6 * (size_t)nat); b.shift = cv.take<double>(nsh); b.Jq = cv.take<double>(nsh);
    b.vs = cv.take<double>(nat); b.vd = cv.take<double>(3 * (size_t)nat); b.vq = cv.take<double>(6 * (size_t)nat);
    b.radcn = cv.take<double>(nat);
    const size_t nr = (size_t)nat * MAXREF;
    b.gw = cv.take<double>(nr); b.dgw = cv.take<double>(nr); b.zeta = cv.take<double>(nr);
    b.dzeta = cv.take<double>(nr); b.Wz = cv.take<double>(nr); b.zv = cv.take<double>(nr); b.zr = cv.take<double>(nr);
    b.zdcn = cv.take<double>(nr); b.zrdcn = cv.take<double>(nr);
    b.vat = cv.take<double>(nat); b.ed4 = cv.take<double>(nat); b.eh0 = cv.take<double>(nat);
    b.eaes = cv.take<double>(2 * (size_t)nat); b.erep = cv.take<double>(nat); b.e2 = cv.take<double>(nat);
    b.e3 = cv.take<double>(aa / 2 + nat + 1); b.grad = cv.take<double>(3 * (size_t)nat);
    b.dhdcn = cv.take<double>(nat); b.tmp2 = cv.take<double>(nat); b.rows = cv.take<double>((size_t)nao * 12);
    b.emo = cv.take<double>(nao); b.focc = cv.take<double>(nao); b.focca = cv.take<double>(nao);
    b.foccb = cv.take<double>(nao); b.fe = cv.take<double>(nao); b.tri_d = cv.take<double>(nao);
    b.tri_e = cv.take<double>(nao); b.tri_e2 = cv.take<double>(nao); b.tri_tau = cv.take<double>(nao);
    b.tri_p = cv.take<double>(2 * (size_t)nao); b.bounds = cv.take<double>(8);
    b.fscal = cv.take<double>(8); b.escal = cv.take<double>(16); b.rms = cv.take<double>(4);
    const int nbr = nsh + 9 * nat;
    b.qin = cv.take<double>(nbr); b.qout = cv.take<double>(nbr); b.dq = cv.take<double>(nbr);
    b.kocc = cv.take<int>(4);
    BroydenState& bs = b.bs;
    bs.nbr = nbr;
    bs.maxit = BATCH_HIST;
    bs.df = cv.take<double>((size_t)BATCH_HIST * nbr);
    bs.u = cv.take<double>((size_t)BATCH_HIST * nbr);
    bs.a = cv.take<double>((size_t)BATCH_HIST * BATCH_HIST);
    bs.omega = cv.take<double>(BATCH_HIST);
    bs.qlast = cv.take<double>(nbr);
    bs.dqlast = cv.take<double>(nbr);
    bs.scratch = cv.take<double>(2 * (size_t)BATCH_HIST * BATCH_HIST + 2 * (size_t)BATCH_HIST + 64);
    b.nel_a = hm.nel_a;
    b.nel_b = hm.nel_b;
    b.charge = hm.charge;
    b.stage = BS_SETUP;
    b.iter = 0;
    b.lastdiag = 0;
    b.converged = 0;
    b.status = BST_OK;
    b.eel = 0.0;
    b.eold = 0.0;
    for (double& o : b.out) o = 0.0;
}

}  // namespace

// ------------------------------------------------------------------ device program of one molecule
#define CTA_FOR(i, n) for (int i = threadIdx.x; i < (n); i += blockDim.x)
#define CTA_FORL(i, n) for (long i = threadIdx.x; i < (long)(n); i += blockDim.x)
#define WARP_FOR(i, n) for (int i = (int)(threadIdx.x >> 5); i < (n); i += (int)(blockDim.x >> 5))

struct DevThresh {
    double intcut, neglect, scfconv, qconv;
};

// thresholds of the reference (src/scf_module.F90:266-277), computed on the host
DevThresh thresholds(double acc) {
    DevThresh t;
    t.intcut = std::max(20.0, 25.0 - 10.0 * std::log10(acc));
    t.neglect = 10.0e-9 * acc;
    t.scfconv = 1.0e-6 * acc;
    t.qconv = 1.0e-4 * acc;
    return t;
}

__device__ void blk_zero(double* p, size_t n) {
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) p[i] = 0.0;
}

// set-up: CN, self energies, EEQ guess, repulsion, integrals, Coulomb/AES/D4 kernels, X = U^-1
__device__ void stage_setup_a(BatchMol* b) {
    const DevMol m = b->m;
    const int nat = m.nat, nsh = m.nsh, nao = m.nao;
    const size_t nn = (size_t)nao * nao;
    blk_zero(b->grad, 3 * (size_t)nat);
    blk_zero(b->dhdcn, nat);
    CTA_FOR(a, nat) d_cn(m, 0, b->cn_gfn, a);
    __syncthreads();
    CTA_FOR(s, nsh) b->se[s] = m.sh_se0[s] - m.sh_kcn[s] * b->cn_gfn[m.sh_atom[s]];
    if (b->guess) {
        // given initial wavefunction (warm start): [qsh; per atom (dipm 3, qp 6)] as packed for mixing
        const int nbr = nsh + 9 * nat;
        CTA_FOR(t, nbr) b->qin[t] = b->guess[t];
        __syncthreads();
        CTA_FOR(t, max(nsh, nat)) d_broyden_unpack(m, b->qin, b->qsh, b->dipm, b->qp, b->q, t);
        __syncthreads();
    } else {
    // EEQ guess (src/eeq_model.f90), iniqshell
    CTA_FOR(a, nat) d_cn(m, 2, b->cn_tmp, a);
    __syncthreads();
    CTA_FORL(t, (long)nat * nat) d_eeq_matrix(m, b->cn_tmp, b->eeqA, b->eeqX, t);
    __syncthreads();
    const int einfo = cta_potrf_upper(nat, b->eeqA, nat);
    d_eeq_solve(nat, b->eeqA, b->eeqX, b->charge, b->q);
    __syncthreads();
    if (einfo != 0) CTA_FOR(a, nat) b->q[a] = b->charge / nat;
    __syncthreads();
    CTA_FOR(s, nsh) b->qsh[s] = m.sh_zsh[s] / b->zval[m.sh_atom[s]] * b->q[m.sh_atom[s]];
    blk_zero(b->dipm, 3 * (size_t)nat);
    blk_zero(b->qp, 6 * (size_t)nat);
    __syncthreads();
    CTA_FOR(t, max(nsh, nat)) d_broyden_pack(m, b->qsh, b->dipm, b->qp, b->qin, t);
    __syncthreads();
    CTA_FOR(t, max(nsh, nat)) d_broyden_unpack(m, b->qin, b->qsh, b->dipm, b->qp, b->q, t);
    __syncthreads();
    }
    CTA_FOR(a, nat) d_repulsion(m, b->erep, b->grad, a);
    // integrals: zeroed here, filled by the batched integral kernels between the two set-up halves
    blk_zero(b->S, nn);
    blk_zero(b->H0, nn);
    blk_zero(b->D, 3 * nn);
    blk_zero(b->Q, 6 * nn);
    __syncthreads();
}

// set-up, second half (after the integrals): Coulomb/AES/D4 kernels, S = U^T U, X = U^-1
__device__ void stage_setup_b(BatchMol* b) {
    const DevMol m = b->m;
    const int nat = m.nat, nsh = m.nsh, nao = m.nao;
    const size_t nn = (size_t)nao * nao;
    CTA_FOR(a, nat) d_radcn(m, b->cn_gfn, b->radcn, a);
    CTA_FORL(t, (long)nsh * nsh) d_jmat(m, b->J, t);
    CTA_FOR(a, nat) d_cn(m, 3, b->cn_tmp, a);
    __syncthreads();
    CTA_FORL(t, (long)nat * nat) d_gab(m, b->radcn, b->gab3, b->gab5, t);
    CTA_FOR(a, nat) d_d4_weights(m, b->cn_tmp, b->gw, nullptr, a);
    // S = U^T U, X = U^-1
    for (size_t i = threadIdx.x; i < nn; i += blockDim.x) b->T1[i] = b->S[i];
    __syncthreads();
    const int sinfo = cta_potrf_upper(nao, b->T1, nao);
    WARP_FOR(j, nao) d_trinv_col(nao, b->T1, nao, b->X, nao, j, threadIdx.x & 31);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (sinfo != 0) {
            b->status = BST_CHOLESKY;
            b->stage = BS_DONE;
        } else {
            b->stage = BS_SCC;
        }
    }
    __syncthreads();
}

// D4 charge scaling, W zeta, atomic potential and energy (d4_scc of the plain engine)
__device__ void d4_scc_blk(BatchMol* b) {
    const DevMol m = b->m;
    CTA_FOR(a, m.nat) d_d4_zeta(m, b->gw, b->q, b->zeta, b->dzeta, a);
    __syncthreads();
    WARP_FOR(a, m.nat) d_d4_wz(m, b->gw, b->zeta, b->dzeta, b->Wz, b->vat, b->ed4, a, threadIdx.x & 31);
    __syncthreads();
}

// SCC energy from the current populations (same sums as the plain engine)
__device__ void scc_energy_blk(BatchMol* b) {
    __shared__ double red[32];
    const DevMol m = b->m;
    double es = 0.0, h = 0.0, ea = 0.0, ep = 0.0, ed = 0.0;
    CTA_FOR(s, m.nsh) es += 0.5 * b->qsh[s] * b->Jq[s] + m.sh_gam3[s] * b->qsh[s] * b->qsh[s] * b->qsh[s] / 3.0;
    CTA_FOR(a, m.nat) {
        h += b->eh0[a];
        ea += b->eaes[a];
        ep += b->eaes[m.nat + a];
        ed += b->ed4[a];
    }
    es = block_sum(es, red);
    h = block_sum(h, red);
    ea = block_sum(ea, red);
    ep = block_sum(ep, red);
    ed = block_sum(ed, red);
    if (threadIdx.x == 0) {
        const double ts = b->fscal[0];
        b->escal[0] = es + h * EVTOAU + ea + ep + ed + ts;
        b->escal[1] = es;
        b->escal[2] = ea;
        b->escal[3] = ep;
        b->escal[4] = ed;
        b->escal[5] = ts;
    }
    __syncthreads();
}

// One SCC iteration (the body of the plain engine's loop); updates the convergence state.
// `sm` is dynamic shared memory of max((4 + 8) * nao + 32, GEMM_SMEM) doubles.
__device__ void scc_iteration(BatchMol* b, const DevThresh& th, double etemp, int maxiter, double* sm) {
    const DevMol m = b->m;
    const int nat = m.nat, nsh = m.nsh, nao = m.nao;
    const size_t nn = (size_t)nao * nao;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int it = b->iter + 1;
    // potentials and H
    d4_scc_blk(b);
    WARP_FOR(s, nsh) d_shell_shift(m, b->J, b->qsh, b->vat, b->shift, b->Jq, s, lane);
    WARP_FOR(i, nat) d_aes_pot(m, b->q, b->dipm, b->qp, b->gab3, b->gab5, 1, b->vs, b->vd, b->vq, i, lane);
    __syncthreads();
    // Hu: upper triangle of H with half its diagonal (H = Hu + Hu^T)
    for (size_t t = threadIdx.x; t < nn; t += blockDim.x) {
        const int i = (int)(t / nao), j = (int)(t % nao);
        if (i > j) {
            b->H[t] = 0.0;
            continue;
        }
        d_build_h(m, th.neglect, b->H0, b->S, b->D, b->Q, b->shift, b->vs, b->vd, b->vq, b->H, t);
        if (i == j) b->H[t] *= 0.5;
    }
    __syncthreads();
    // A = X^T H X = B + B^T with B = X^T (Hu X): n^3 flops against 5/3 n^3 for X^T (H X)
    cta_dgemm<false, false>(nao, nao, nao, 1.0, b->H, nao, b->X, nao, 0.0, b->T1, nao, GF_A_UPPER | GF_B_UPPER, nullptr,
                            nullptr, sm);
    cta_dgemm<true, false>(nao, nao, nao, 1.0, b->X, nao, b->T1, nao, 0.0, b->A, nao, GF_A_LOWER | GF_B_UPPER, nullptr,
                           nullptr, sm);
    for (size_t t = threadIdx.x; t < nn; t += blockDim.x) {
        const int i = (int)(t / nao), j = (int)(t % nao);
        if (i < j) continue;
        const size_t tt = (size_t)j * nao + i;
        if (i == j) {
            b->A[t] *= 2.0;
        } else {
            const double s = b->A[t] + b->A[tt];
            b->A[t] = s;
            b->A[tt] = s;
        }
    }
    __syncthreads();
    // eigenvalues, occupations, occupied eigenvectors
    d_sytrd<true>(nao, b->A, nao, b->V, b->tri_tau, b->tri_d, b->tri_e, b->tri_p, sm);
    __syncthreads();
    d_tri_prep(nao, b->tri_d, b->tri_e, b->tri_e2, b->bounds);
    __syncthreads();
    stage_tridiag(nao, b->tri_d, b->tri_e2, sm);
    __syncthreads();
    // levels ja .. jb - 1 by multisection
    auto bisect_levels = [&](int ja, int jb) {
        const float* fsm = reinterpret_cast<const float*>(sm + 2 * nao);
        const int per_pass = (int)(blockDim.x / BIS_G);
        for (int j0 = ja; j0 < jb; j0 += per_pass) {   // uniform trip count: whole warps stay together
            const int j = j0 + (int)(threadIdx.x / BIS_G);
            const bool valid = j < jb;
            const double v = d_bisect_group<true>(nao, sm, sm + nao, fsm, fsm + nao, b->bounds, valid ? j : 0, valid);
            if (valid && threadIdx.x % BIS_G == 0) b->emo[j] = v;
        }
    };
    // inside the SCC only the levels that can carry occupation: the lowest nocc + max(8, n / 8),
    // the rest (with a second smearing) only when the last of them lies less than 60 kT above a
    // Fermi level (the smearing is exactly zero from 50 kT); the last diagonalisation takes all
    const int klev = (b->lastdiag || it >= maxiter) ? nao : min(nao, max(b->nel_a, b->nel_b) + max(8, nao / 8));
    bisect_levels(0, klev);
    for (int j = klev + (int)threadIdx.x; j < nao; j += (int)blockDim.x) b->emo[j] = 1.0e300;
    __syncthreads();
    d_fermi(nao, b->emo, b->nel_a, b->nel_b, etemp, b->focc, b->focca, b->foccb, b->fscal, b->kocc);
    __syncthreads();
    if (klev < nao &&
        b->emo[klev - 1] - fmax(b->fscal[1], b->fscal[2]) < 60.0 * KB_AU * AUTOEV * etemp) {   // block-uniform
        bisect_levels(klev, nao);
        __syncthreads();
        d_fermi(nao, b->emo, b->nel_a, b->nel_b, etemp, b->focc, b->focca, b->foccb, b->fscal, b->kocc);
        __syncthreads();
    }
    const int kocc = *b->kocc;
    double* U1 = b->iscr;
    CTA_FOR(j, kocc) d_inviter<2>(nao, b->tri_d, b->tri_e, b->emo, b->bounds, b->Y, U1, U1 + nn, U1 + 2 * nn,
                               U1 + 3 * nn, b->piv, j);
    __syncthreads();
    WARP_FOR(j, kocc) d_reorth(nao, b->emo, b->bounds, 1.0e-7, b->Y, U1, U1 + nn, U1 + 2 * nn, U1 + 3 * nn, b->piv,
                               kocc, j, lane);
    __syncthreads();
    // Z = Q Y: one occupied column per lane, 32 per warp
    for (int g = wid; g * 32 < kocc; g += (int)(blockDim.x >> 5)) d_ormtr_cols(nao, b->V, b->tri_tau, b->Y, b->Zt, g * 32, kocc, lane);
    __syncthreads();
    // C = X Z, P = C f C^T
    cta_dgemm<false, true>(nao, nao, nao, 1.0, b->X, nao, b->Zt, nao, 0.0, b->C, nao, GF_A_UPPER, nullptr, b->kocc, sm);
    for (size_t t = threadIdx.x; t < nn; t += blockDim.x) d_scale_cols(nao, b->C, b->focc, b->T1, t);
    __syncthreads();
    cta_dgemm<false, true>(nao, nao, nao, 1.0, b->T1, nao, b->C, nao, 0.0, b->P, nao, GF_SYM, b->kocc, nullptr, sm);
    cta_mirror_lower(nao, b->P, nao);
    // populations, energies, mixing
    CTA_FOR(mu, nao) d_rowsums_thread(m, b->P, b->S, b->D, b->Q, b->H0, b->rows, mu);
    __syncthreads();
    CTA_FOR(a, nat) d_atom_pop(m, b->rows, b->qsh, b->q, b->dipm, b->qp, b->eh0, a);
    __syncthreads();
    WARP_FOR(s, nsh) d_shell_shift(m, b->J, b->qsh, nullptr, b->T1, b->Jq, s, lane);
    WARP_FOR(i, nat) d_aes_energy(m, b->q, b->dipm, b->qp, b->gab3, b->gab5, b->eaes, i, lane);
    __syncthreads();
    d4_scc_blk(b);
    scc_energy_blk(b);
    CTA_FOR(t, max(nsh, nat)) d_broyden_pack(m, b->qsh, b->dipm, b->qp, b->qout, t);
    __syncthreads();
    const BroydenState& bs = b->bs;
    d_broyden(bs.nbr, it, bs.maxit, 0.4, b->qin, b->qout, b->dq, bs.df, bs.u, bs.a, bs.omega, bs.qlast, bs.dqlast,
              bs.scratch, b->rms, nat);
    __syncthreads();
    CTA_FOR(t, max(nsh, nat)) d_broyden_unpack(m, b->qin, b->qsh, b->dipm, b->qp, b->q, t);
    __syncthreads();
    if (threadIdx.x == 0) {
        b->iter = it;
        b->eold = b->eel;
        b->eel = b->escal[0];
        const bool econv = fabs(b->eel - b->eold) < th.scfconv;
        const bool qconvd = b->rms[0] < th.qconv;
        if (!isfinite(b->eel)) {
            b->status = BST_NONFINITE;
            b->stage = BS_DONE;
        } else {
            bool stop = false;
            if (econv && qconvd) {
                b->converged = 1;
                if (b->lastdiag) stop = true;
                b->lastdiag = 1;
            }
            if (!stop && it >= maxiter) {
                stop = true;
                if (!b->converged) b->status = BST_NOT_CONVERGED;
            }
            if (!stop && it >= BATCH_HIST + 1) {   // out of Broyden history: hand over to the plain engine
                b->status = BST_HISTORY;
                b->stage = BS_DONE;
            } else if (stop) {
                b->stage = BS_GRAD;
            }
        }
    }
    __syncthreads();
}

// Gradient, dipole and energy assembly (the plain engine after its SCC loop).
__device__ void stage_gradient_a(BatchMol* b, double* sm) {
    const DevMol m = b->m;
    const int nat = m.nat, nao = m.nao;
    const size_t nn = (size_t)nao * nao;
    const int lane = threadIdx.x & 31;
    const bool want_grad = b->want_grad != 0;
    if (want_grad) {
        CTA_FOR(i, nao) b->fe[i] = b->focc[i] * b->emo[i] * EVTOAU;
        __syncthreads();
        for (size_t t = threadIdx.x; t < nn; t += blockDim.x) d_scale_cols(nao, b->C, b->fe, b->T1, t);
        __syncthreads();
        cta_dgemm<false, true>(nao, nao, nao, 1.0, b->T1, nao, b->C, nao, 0.0, b->W, nao, GF_SYM, b->kocc, nullptr, sm);
        cta_mirror_lower(nao, b->W, nao);
        WARP_FOR(i, nat) d_aes_pot(m, b->q, b->dipm, b->qp, b->gab3, b->gab5, 0, b->vs, b->vd, b->vq, i, lane);
        __syncthreads();
    }
}

// gradient, second half (after the integral-derivative kernels)
__device__ void stage_gradient_b(BatchMol* b) {
    __shared__ double red[32];
    const DevMol m = b->m;
    const int nat = m.nat, nao = m.nao;
    const int lane = threadIdx.x & 31;
    const bool want_grad = b->want_grad != 0;
    if (want_grad) {
        CTA_FOR(a, nat) d_dhdcn_diag(m, b->P, b->dhdcn, a);
        __syncthreads();
        WARP_FOR(i, nat) d_aes_grad(m, b->q, b->dipm, b->qp, b->radcn, b->gab3, b->gab5, b->grad, b->tmp2, i, lane);
        __syncthreads();
        CTA_FOR(a, nat) d_aes_dradcn(m, b->cn_gfn, b->tmp2, b->dhdcn, a);
        __syncthreads();
        CTA_FOR(a, nat) d_cn_chain(m, 0, b->dhdcn, b->grad, a);
        __syncthreads();
    }
    // D4 two-body and ATM at the final charges, covalent CN (energy always, gradient on request)
    CTA_FOR(a, nat) {
        d_cn(m, 1, b->cn_tmp, a);
        b->tmp2[a] = 0.0;
    }
    __syncthreads();
    CTA_FOR(a, nat) d_d4_weights(m, b->cn_tmp, b->gw, b->dgw, a);
    __syncthreads();
    CTA_FOR(a, nat) d_d4_refvec(m, b->gw, b->dgw, b->q, b->zv, b->zr, b->zdcn, b->zrdcn, a);
    __syncthreads();
    CTA_FORL(t, (long)nat * nat) {
        d_d4_c6(m, b->zv, b->zdcn, b->c6, b->dc6, t);
        d_d4_c6(m, b->zr, b->zrdcn, b->c6z, b->dc6z, t);
    }
    __syncthreads();
    // (without a gradient request the gradient terms land in b->grad and are not reported)
    CTA_FOR(a, nat) d_d4_2body(m, b->c6, b->dc6, b->e2, b->tmp2, b->grad, a);
    __syncthreads();
    const long npa = (long)nat * (nat + 1) / 2;
    CTA_FORL(t, npa) d_d4_atm(m, b->c6z, b->dc6z, npa, b->e3, b->tmp2, b->grad, t);
    __syncthreads();
    if (want_grad) {
        CTA_FOR(a, nat) d_cn_chain(m, 1, b->tmp2, b->grad, a);
        __syncthreads();
        WARP_FOR(a, nat) d_coulomb_grad(m, b->qsh, b->grad, a, lane);
        __syncthreads();
    }
    // dipole (calc_dipole, src/dipole.f90:94-128)
    double dip[3];
    for (int k = 0; k < 3; ++k) {
        double s = 0.0;
        CTA_FOR(a, nat) s += m.xyz[3 * a + k] * b->zval[a];
        CTA_FOR(mu, nao) s -= b->rows[(size_t)mu * 12 + 1 + k];
        dip[k] = block_sum(s, red);
    }
    // repulsion and three-body sums in the plain engine's order
    double er = 0.0, e3 = 0.0;
    CTA_FOR(a, nat) er += b->erep[a];
    er = block_sum(er, red);
    CTA_FORL(t, npa) e3 += b->e3[t];
    e3 = block_sum(e3, red);
    if (threadIdx.x == 0) {
        double* o = b->out;
        o[BO_REP] = er;
        o[BO_ATM] = e3;
        o[BO_ENERGY] = b->eel + er + e3;
        o[BO_ELEC] = b->eel + e3;
        o[BO_ES] = b->escal[1];
        o[BO_AES] = b->escal[2];
        o[BO_AXC] = b->escal[3];
        o[BO_DISP] = b->escal[4] + e3;
        const int ih = b->nel_a;
        o[BO_GAP] = (ih >= 1 && ih < nao) ? (b->emo[ih] - b->emo[ih - 1]) : 0.0;
        o[BO_DIPX] = dip[0];
        o[BO_DIPY] = dip[1];
        o[BO_DIPZ] = dip[2];
        b->stage = BS_DONE;
    }
    __syncthreads();
}

// One block per molecule; a block whose molecule is not in the kernel's stage exits at once.
__device__ __forceinline__ BatchMol* mol_in_stage(BatchMol* mols, int nmol, int stage) {
    const int mi = blockIdx.x;
    if (mi >= nmol) return nullptr;
    BatchMol* b = mols + mi;
    return (b->stage == stage) ? b : nullptr;
}

__global__ void __launch_bounds__(BT) k_batch_setup_a(BatchMol* __restrict__ mols, int nmol) {
    BatchMol* b = mol_in_stage(mols, nmol, BS_SETUP);
    if (b) stage_setup_a(b);
}

__global__ void __launch_bounds__(BT) k_batch_setup_b(BatchMol* __restrict__ mols, int nmol) {
    BatchMol* b = mol_in_stage(mols, nmol, BS_SETUP);
    if (b) stage_setup_b(b);
}

// up to max_iter SCC iterations of every molecule in the SCC stage
// four molecules per SM (at most 64 registers): the SCC's dependent FP64 chains and shared-
// memory round trips need the other blocks' warps to hide them (3502 single points/s at two per
// SM, 3608 at three, 3735 at four with a few hundred bytes of spills, no more at five)
__global__ void __launch_bounds__(BT, 4) k_batch_scc(BatchMol* __restrict__ mols, int nmol, DevThresh th, double etemp,
                                                  int maxiter, int max_iter) {
    extern __shared__ double sm[];
    BatchMol* b = mol_in_stage(mols, nmol, BS_SCC);
    if (!b) return;
    __shared__ int stage;
    stage = BS_SCC;
    __syncthreads();
    for (int k = 0; k < max_iter && stage == BS_SCC; ++k) {
        scc_iteration(b, th, etemp, maxiter, sm);
        if (threadIdx.x == 0) stage = b->stage;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(BT) k_batch_grad_a(BatchMol* __restrict__ mols, int nmol) {
    __shared__ double sm[GEMM_SMEM];
    BatchMol* b = mol_in_stage(mols, nmol, BS_GRAD);
    if (b) stage_gradient_a(b, sm);
}

__global__ void __launch_bounds__(BT) k_batch_grad_b(BatchMol* __restrict__ mols, int nmol) {
    BatchMol* b = mol_in_stage(mols, nmol, BS_GRAD);
    if (b) stage_gradient_b(b);
}

// Pack the per-molecule gradient [nat][3] and charges [nat] into contiguous outputs
// (atom offset off[mi]); one block per molecule.
__global__ void k_batch_gather(const BatchMol* __restrict__ mols, int nmol, const long* __restrict__ off,
                               double* __restrict__ grad, double* __restrict__ q) {
    const int mi = blockIdx.x;
    if (mi >= nmol) return;
    const BatchMol* b = mols + mi;
    const int nat = b->m.nat;
    const long o = off[mi];
    for (int t = threadIdx.x; t < 3 * nat; t += blockDim.x) grad[3 * o + t] = b->grad[t];
    for (int t = threadIdx.x; t < nat; t += blockDim.x) q[o + t] = b->q[t];
}

// ------------------------------------------------------------------ host side
// Upload the recorded parameter arrays to base + offset, merged into contiguous runs
// (the work arrays between them are small gaps); returns the bytes copied.
long long upload_runs(const std::vector<Carver::Up>& ups, char* base, cudaStream_t st) {
    long long bytes = 0;
    std::vector<char> stage;
    size_t i = 0;
    while (i < ups.size()) {
        size_t j = i, lo = ups[i].off, hi = ups[i].off + ups[i].bytes;
        while (j + 1 < ups.size() && ups[j + 1].off - hi < 4096) {
            ++j;
            hi = ups[j].off + ups[j].bytes;
        }
        stage.assign(hi - lo, 0);
        for (size_t k = i; k <= j; ++k) std::memcpy(stage.data() + (ups[k].off - lo), ups[k].src, ups[k].bytes);
        XG_CUDA(cudaMemcpyAsync(base + lo, stage.data(), hi - lo, cudaMemcpyHostToDevice, st));
        XG_CUDA(cudaStreamSynchronize(st));
        bytes += (long long)(hi - lo);
        i = j + 1;
    }
    return bytes;
}

DeviceBatch::~DeviceBatch() {
    if (base_) cudaFree(base_);
}

size_t DeviceBatch::bytes_for(const HostMol& hm) {
    Carver cv;
    BatchMol b{};
    layout_mol(cv, hm, b);
    return cv.used;
}

void DeviceBatch::load(const std::vector<const HostMol*>& mols, const std::vector<int>& want_grad, cudaStream_t st,
                       const std::vector<const Wavefunction*>* guesses) {
    // packed initial wavefunctions [qsh; per atom (dipm 3, qp 6)]
    std::vector<std::vector<double>> packed(mols.size());
    std::vector<const std::vector<double>*> gp(mols.size(), nullptr);
    if (guesses)
        for (size_t i = 0; i < mols.size(); ++i) {
            const Wavefunction* w = (*guesses)[i];
            if (!w || w->nat != mols[i]->nat || w->nsh != mols[i]->nsh) continue;
            auto& v = packed[i];
            v.assign(w->qsh.begin(), w->qsh.end());
            for (int a = 0; a < w->nat; ++a) {
                for (int k = 0; k < 3; ++k) v.push_back(w->dipm[3 * a + k]);
                for (int k = 0; k < 6; ++k) v.push_back(w->qp[6 * a + k]);
            }
            gp[i] = &v;
        }
    nmol_ = (int)mols.size();
    h_mols_.assign(nmol_, BatchMol{});
    max_nao_ = 1;
    max_nsh_ = 1;
    // pass 1: sizes
    Carver cv;
    const size_t desc = ((sizeof(BatchMol) * std::max(nmol_, 1) + 255) / 256) * 256;
    cv.used = desc;
    for (int i = 0; i < nmol_; ++i) {
        if (mols[i]->nao > BATCH_MAX_NAO) throw CudaError("batched engine: molecule exceeds the AO limit");
        layout_mol(cv, *mols[i], h_mols_[i], gp[i]);
        max_nao_ = std::max(max_nao_, mols[i]->nao);
        max_nsh_ = std::max(max_nsh_, mols[i]->nsh);
    }
    const size_t need = cv.used;
    if (need > bytes_) {
        if (base_) cudaFree(base_);
        base_ = nullptr;
        bytes_ = 0;
        XG_CUDA(cudaMalloc(&base_, need));
        bytes_ = need;
    }
    // pass 2: pointers, and the staged parameter upload
    std::vector<Carver::Up> ups;
    h2d_ = (long long)(sizeof(BatchMol) * nmol_);
    Carver cv2;
    cv2.base = base_;
    cv2.used = desc;
    cv2.ups = &ups;
    for (int i = 0; i < nmol_; ++i) {
        layout_mol(cv2, *mols[i], h_mols_[i], gp[i]);
        h_mols_[i].want_grad = want_grad.empty() ? 1 : want_grad[i];
    }
    d_mols_ = reinterpret_cast<BatchMol*>(base_);
    h2d_ += upload_runs(ups, base_, st);
    XG_CUDA(cudaMemcpyAsync(d_mols_, h_mols_.data(), sizeof(BatchMol) * nmol_, cudaMemcpyHostToDevice, st));
    XG_CUDA(cudaStreamSynchronize(st));
}

// The seven launches of one step over `nmol` slots.
void launch_step(BatchMol* d_mols, int nmol, int max_nao, int max_nsh, const BatchSettings& set, int max_iter,
                 cudaStream_t st, cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr) {
    const size_t smem = (size_t)std::max(12 * max_nao + 32, GEMM_SMEM) * sizeof(double);
    if (smem > 48 * 1024) allow_max_dynamic_smem((const void*)k_batch_scc);
    const DevThresh th = thresholds(set.accuracy);
    k_batch_setup_a<<<nmol, BT, 0, st>>>(d_mols, nmol);
    XG_LAUNCH_CHECK();
    batch_integrals(st, d_mols, nmol, max_nsh, th.intcut);
    k_batch_setup_b<<<nmol, BT, 0, st>>>(d_mols, nmol);
    XG_LAUNCH_CHECK();
    if (ev0) XG_CUDA(cudaEventRecord(ev0, st));
    k_batch_scc<<<nmol, BT, smem, st>>>(d_mols, nmol, th, set.etemp, std::max(1, set.maxiter), max_iter);
    XG_LAUNCH_CHECK();
    if (ev1) XG_CUDA(cudaEventRecord(ev1, st));
    k_batch_grad_a<<<nmol, BT, 0, st>>>(d_mols, nmol);
    XG_LAUNCH_CHECK();
    batch_integral_gradient(st, d_mols, nmol, max_nsh, th.intcut);
    k_batch_grad_b<<<nmol, BT, 0, st>>>(d_mols, nmol);
    XG_LAUNCH_CHECK();
}

int DeviceBatch::step(const BatchSettings& set, int max_iter, cudaStream_t st) {
    if (nmol_ == 0) return 0;
    launch_step(d_mols_, nmol_, max_nao_, max_nsh_, set, max_iter, st);
    return nmol_;
}

void DeviceBatch::fetch_states(std::vector<BatchMol>& mols, cudaStream_t st) const {
    mols.resize(nmol_);
    if (nmol_ == 0) return;
    XG_CUDA(cudaMemcpyAsync(mols.data(), d_mols_, sizeof(BatchMol) * nmol_, cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaStreamSynchronize(st));
}

void DeviceBatch::gather(const long* d_off, double* d_grad, double* d_q, cudaStream_t st) const {
    if (nmol_ == 0) return;
    k_batch_gather<<<nmol_, 128, 0, st>>>(d_mols_, nmol_, d_off, d_grad, d_q);
    XG_LAUNCH_CHECK();
}

// ------------------------------------------------------------------ slot pool
SlotPool::SlotPool(size_t budget_bytes, int max_slots) : max_slots_(std::max(1, max_slots)) {
    desc_ = ((sizeof(BatchMol) * max_slots_ + 255) / 256) * 256;
    cap_ = std::max(budget_bytes, desc_ + 4096);
    XG_CUDA(cudaMalloc(&base_, cap_));
    d_slots_ = reinterpret_cast<BatchMol*>(base_);
    std::vector<BatchMol> empty(max_slots_);
    for (auto& b : empty) {
        b = BatchMol{};
        b.stage = BS_DONE;
    }
    XG_CUDA(cudaMemcpy(d_slots_, empty.data(), sizeof(BatchMol) * max_slots_, cudaMemcpyHostToDevice));
    slot_off_.assign(max_slots_, 0);
    slot_size_.assign(max_slots_, 0);
    slot_nao_.assign(max_slots_, 0);
    slot_nsh_.assign(max_slots_, 0);
    slot_iter_.assign(max_slots_, 0);
    slot_nocc_.assign(max_slots_, 0);
    XG_CUDA(cudaEventCreate(&ev0_));
    XG_CUDA(cudaEventCreate(&ev1_));
    free_.push_back({desc_, cap_ - desc_});
}

SlotPool::~SlotPool() {
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (base_) cudaFree(base_);
}

size_t SlotPool::free_bytes() const {
    size_t f = 0;
    for (auto& r : free_) f += r.second;
    return f;
}

int SlotPool::admit(const HostMol& hm, int want_grad, cudaStream_t st) {
    if (hm.nao > BATCH_MAX_NAO) return -1;
    int slot = -1;
    for (int i = 0; i < max_slots_; ++i)
        if (slot_size_[i] == 0) {
            slot = i;
            break;
        }
    if (slot < 0) return -1;
    const size_t need = DeviceBatch::bytes_for(hm);
    size_t k = 0;
    while (k < free_.size() && free_[k].second < need) ++k;
    if (k == free_.size()) return -1;
    const size_t off = free_[k].first;
    free_[k].first += need;
    free_[k].second -= need;
    if (free_[k].second == 0) free_.erase(free_.begin() + k);
    BatchMol b{};
    std::vector<Carver::Up> ups;
    Carver cv;
    cv.base = base_ + off;
    cv.ups = &ups;
    layout_mol(cv, hm, b);
    b.want_grad = want_grad;
    try {
        if (fail_admissions_ > 0) {
            --fail_admissions_;
            throw CudaError("admission failed: out of device memory (injected)");
        }
        h2d_ += upload_runs(ups, base_ + off, st);
        XG_CUDA(cudaMemcpyAsync(d_slots_ + slot, &b, sizeof(BatchMol), cudaMemcpyHostToDevice, st));
        XG_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        // hand the region back, so a failed admission costs only its own request
        std::pair<size_t, size_t> r{off, need};
        free_.insert(std::lower_bound(free_.begin(), free_.end(), r), r);
        for (size_t k = 0; k + 1 < free_.size();) {
            if (free_[k].first + free_[k].second == free_[k + 1].first) {
                free_[k].second += free_[k + 1].second;
                free_.erase(free_.begin() + k + 1);
            } else {
                ++k;
            }
        }
        throw;
    }
    h2d_ += sizeof(BatchMol);
    slot_off_[slot] = off;
    slot_size_[slot] = need;
    slot_nao_[slot] = hm.nao;
    slot_nsh_[slot] = hm.nsh;
    slot_iter_[slot] = 0;
    slot_nocc_[slot] = (hm.nel_a + hm.nel_b + 1) / 2;
    ++resident_;
    hi_ = std::max(hi_, slot + 1);
    return slot;
}

void SlotPool::step(const BatchSettings& set, int max_iter, cudaStream_t st) {
    if (resident_ == 0) return;
    int max_nao = 1, max_nsh = 1;
    for (int i = 0; i < hi_; ++i)
        if (slot_size_[i]) {
            max_nao = std::max(max_nao, slot_nao_[i]);
            max_nsh = std::max(max_nsh, slot_nsh_[i]);
        }
    launch_step(d_slots_, hi_, max_nao, max_nsh, set, max_iter, st, ev0_, ev1_);
}

void SlotPool::finished(std::vector<int>& slots, std::vector<BatchMol>& states, cudaStream_t st) {
    slots.clear();
    states.clear();
    if (resident_ == 0) return;
    std::vector<BatchMol> all(hi_);
    XG_CUDA(cudaMemcpyAsync(all.data(), d_slots_, sizeof(BatchMol) * hi_, cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaStreamSynchronize(st));
    last_state_bytes_ = sizeof(BatchMol) * hi_;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, ev0_, ev1_) == cudaSuccess) last_ms_ = ms;
    else cudaGetLastError();
    last_flops_ = 0.0;
    for (int i = 0; i < hi_; ++i) {
        if (!slot_size_[i]) continue;
        const double n = slot_nao_[i], k = slot_nocc_[i];
        last_flops_ += (double)(all[i].iter - slot_iter_[i]) * ((16.0 / 3.0) * n * n * n + 2.0 * n * n * k);
        slot_iter_[i] = all[i].iter;
        if (all[i].stage == BS_DONE) {
            slots.push_back(i);
            states.push_back(all[i]);
        }
    }
}

void SlotPool::copy_results(const BatchMol& state, double* grad, double* q, cudaStream_t st) const {
    const int nat = state.m.nat;
    XG_CUDA(cudaMemcpyAsync(grad, state.grad, 3 * sizeof(double) * nat, cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaMemcpyAsync(q, state.q, sizeof(double) * nat, cudaMemcpyDeviceToHost, st));
}

void SlotPool::release(int slot) {
    if (slot < 0 || slot >= max_slots_ || slot_size_[slot] == 0) return;
    // the descriptor on the device keeps stage BS_DONE, so later steps skip the slot
    std::pair<size_t, size_t> r{slot_off_[slot], slot_size_[slot]};
    auto it = std::lower_bound(free_.begin(), free_.end(), r);
    it = free_.insert(it, r);
    if (it + 1 != free_.end() && it->first + it->second == (it + 1)->first) {
        it->second += (it + 1)->second;
        free_.erase(it + 1);
    }
    if (it != free_.begin() && (it - 1)->first + (it - 1)->second == it->first) {
        (it - 1)->second += it->second;
        free_.erase(it);
    }
    slot_size_[slot] = 0;
    --resident_;
    while (hi_ > 0 && slot_size_[hi_ - 1] == 0) --hi_;
}

}  // namespace xg
