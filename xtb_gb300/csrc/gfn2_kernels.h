// Device data layout and launchers of the GFN2-xTB kernels.
#pragma once
#include "common.cuh"

namespace xg {

constexpr int MAXPRIM = 6;
constexpr int MAXREF = 7;

// Per-molecule device arrays (all FP64 unless noted).  AOs of an atom and of a
// shell are contiguous; shells of an atom are contiguous.
struct DevMol {
    int nat = 0, nsh = 0, nao = 0;
    int nelem = 0;                 // number of distinct elements (D4 tables)
    // atoms
    const int* Z = nullptr;        // atomic number
    const int* eid = nullptr;      // element id 0..nelem-1
    const double* xyz = nullptr;   // [nat][3] Bohr
    const int* at_sh0 = nullptr;   // first shell of atom
    const int* at_nsh = nullptr;   // shells of atom
    const int* at_ao0 = nullptr;   // first AO of atom
    const int* at_nao = nullptr;   // AOs of atom
    const double* rcov = nullptr;     // covalentRadD3 (Bohr)
    const double* en = nullptr;       // Pauling EN
    const double* rcov4 = nullptr;    // single-precision D4 radii
    const double* en4 = nullptr;      // single-precision D4 EN
    const double* eeq_en = nullptr, *eeq_gam = nullptr, *eeq_kappa = nullptr, *eeq_alpha = nullptr;
    const double* mrad = nullptr, *valcn = nullptr, *dkern = nullptr, *qkern = nullptr;
    const double* rep_alpha = nullptr, *rep_zeff = nullptr;
    const double* r4r2 = nullptr;     // sqrt(Z r4/r2)
    const double* arad = nullptr;     // atomic radius for the shell polynomial
    // D4 per element id
    const int* d4_nref = nullptr;     // [nelem]
    const double* d4_zeff = nullptr, *d4_gam = nullptr;                 // [nelem]
    const double* d4_refq = nullptr, *d4_refcn = nullptr;               // [nelem][MAXREF]
    const int* d4_ncount = nullptr;                                     // [nelem][MAXREF]
    const double* d4_c6 = nullptr;    // [nelem][nelem][MAXREF][MAXREF]
    // shells
    const int* sh_atom = nullptr, *sh_l = nullptr, *sh_ao = nullptr, *sh_nprim = nullptr;
    const double* sh_alpha = nullptr, *sh_coef = nullptr;   // [nsh][MAXPRIM]
    const double* sh_zeta = nullptr, *sh_se0 = nullptr, *sh_kcn = nullptr, *sh_poly = nullptr;
    const double* sh_eta = nullptr, *sh_gam3 = nullptr, *sh_zsh = nullptr;
    // AOs
    const int* ao_sh = nullptr, *ao_at = nullptr;
    // shells grouped by angular momentum: group l is sh_byl[l_off[l] .. l_off[l + 1])
    const int* sh_byl = nullptr;
    int l_off[4] = {0, 0, 0, 0};
};

struct Thresholds {
    double intcut;    // primitive prefactor cut
    double neglect;   // D/Q list screening threshold
};

// ---- coordination numbers: mode 0 = gfn (k=10), 1 = cov (erf, EN), 2 = erf EEQ (float radii), 3 = d4 (float radii/EN)
void cn(cudaStream_t st, const DevMol& m, int mode, double* cn_out);
// g[a] += sum_b dCN_b/dR_a * v[b]  for modes 0 / 1
void cn_chain(cudaStream_t st, const DevMol& m, int mode, const double* v, double* grad);

// ---- EEQ guess
void eeq_setup(cudaStream_t st, const DevMol& m, const double* cn, double* A /*nat x nat*/, double* X /*2*nat*/);
void eeq_finish(cudaStream_t st, int nat, const double* A_factor, double* X, double charge, double* q, double* work);

// ---- integrals: S, D(3), Q(6) (origin 0) and H0 (eV); se = CN-shifted self energies per shell
void build_sdqh0(cudaStream_t st, const DevMol& m, const double* se, Thresholds th, double* S, double* D, double* Q,
                 double* H0);

// ---- electrostatics setup
void coulomb_matrix(cudaStream_t st, const DevMol& m, double* J);
void aes_setup(cudaStream_t st, const DevMol& m, const double* cn, double* radcn, double* gab3, double* gab5);

// ---- D4
void d4_weights(cudaStream_t st, const DevMol& m, const double* cn, double* gw, double* dgw /*may be null*/);
// Wz[a][r] = sum_b f_ab sum_s gw_ar c6_rs gw_bs zeta_bs (masked exactly like the reference W matrix)
void d4_scc(cudaStream_t st, const DevMol& m, const double* gw, const double* q, double* zeta, double* dzeta,
            double* Wz, double* vat, double* e_atom);

// ---- SCC iteration pieces
void shell_shift(cudaStream_t st, const DevMol& m, const double* J, const double* qsh, const double* vat_d4,
                 double* shift, double* Jq);
void aes_potential(cudaStream_t st, const DevMol& m, const double* q, const double* dipm, const double* qp,
                   const double* gab3, const double* gab5, bool shifted, double* vs, double* vd, double* vq);
// Hu, the upper triangle of the Hamiltonian with half its diagonal (H = Hu + Hu^T); the lower
// triangle is set to zero without being computed
void build_hu(cudaStream_t st, const DevMol& m, Thresholds th, const double* H0, const double* S, const double* D,
              const double* Q, const double* shift, const double* vs, const double* vd, const double* vq, double* H);
// Fermi smearing (one block): focc = fa + fb (alpha, beta occupations), scal = {entropy term, e_fermi_a, e_fermi_b}
// kocc[0] = number of leading orbitals with non-zero occupation
// (only when *gate != 0, if gate is given)
void fermi(cudaStream_t st, int n, const double* emo, int nel_a, int nel_b, double etemp, double* focc, double* fa,
           double* fb, double* scal, int* kocc, const int* gate = nullptr);
// scale columns: Cf[i][j] = C[i][j] * f[j]
void scale_cols(cudaStream_t st, int n, const double* C, const double* f, double* Cf);
// Mulliken + multipole row sums and per-atom/shell reduction
void populations(cudaStream_t st, const DevMol& m, const double* P, const double* S, const double* D, const double* Q,
                 const double* H0, double* rows /*nao*12*/, double* qsh, double* q, double* dipm, double* qp,
                 double* eh0_part /*nat*/);
void aes_energy(cudaStream_t st, const DevMol& m, const double* q, const double* dipm, const double* qp,
                const double* gab3, const double* gab5, double* e_part /*2*nat*/);
// sum of arrays into scalars (one block, deterministic)
void reduce_sum(cudaStream_t st, const double* x, int n, double* out);

// ---- Broyden mixing (modified Broyden, Johnson 1988)
struct BroydenState {
    int nbr = 0, maxit = 0;
    double* df = nullptr;      // [maxit][nbr]
    double* u = nullptr;       // [maxit][nbr]
    double* a = nullptr;       // [maxit][maxit]
    double* omega = nullptr;   // [maxit]
    double* qlast = nullptr;   // [nbr]
    double* dqlast = nullptr;  // [nbr]
    double* scratch = nullptr; // [4*maxit + maxit*maxit*2 + 64]
};
void broyden_pack(cudaStream_t st, const DevMol& m, const double* qsh, const double* dipm, const double* qp, double* vec);
void broyden_unpack(cudaStream_t st, const DevMol& m, const double* vec, double* qsh, double* dipm, double* qp, double* q);
void broyden_step(cudaStream_t st, BroydenState& bs, int it, double alpha, double* qin, const double* qout,
                  double* dq, double* rms_out, int nat);

// ---- gradient
void grad_sdqh0(cudaStream_t st, const DevMol& m, Thresholds th, const double* se, const double* P, const double* Pew,
                const double* shift, const double* vs, const double* vd, const double* vq, double* grad, double* dhdcn);
void dhdcn_diag(cudaStream_t st, const DevMol& m, const double* P, double* dhdcn);
void repulsion(cudaStream_t st, const DevMol& m, double* e_atom, double* grad);
void coulomb_grad(cudaStream_t st, const DevMol& m, const double* qsh, double* grad);
void aes_grad(cudaStream_t st, const DevMol& m, const double* q, const double* dipm, const double* qp,
              const double* radcn, const double* gab3, const double* gab5, double* grad, double* tmp2);
void aes_dradcn(cudaStream_t st, const DevMol& m, const double* cn, const double* tmp2, double* dhdcn);
// D4 dispersion energy and gradient at fixed charges (2-body + ATM); dEdcn accumulated.
// c6 and dc6 are overwritten (ATM pair factors); pair_work: 3 nat^2 doubles of scratch.
void d4_grad(cudaStream_t st, const DevMol& m, const double* cn, const double* q, double* gw, double* dgw,
             double* zv, double* zr, double* zdcn, double* zrdcn, double* c6, double* dc6, double* c6z, double* dc6z, double* e2_atom,
             double* e3_atom, double* dEdcn, double* grad, double* pair_work);
void add_vec(cudaStream_t st, int n, const double* a, double* b);

}  // namespace xg
