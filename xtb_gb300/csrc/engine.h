// Plain per-molecule FP64 GFN2-xTB single point on one GPU (host orchestration).
#pragma once
#include <string>
#include <vector>

#include "host_model.h"
#include "solvation.h"
#include "tune.h"

namespace xg {

struct SPSettings {
    double accuracy = 1.0;     // xtb_setAccuracy
    double etemp = 300.0;      // xtb_setElectronicTemp (K)
    int maxiter = 250;         // xtb_setMaxIter
    // 0: every product in FP64; 1: the back-transformation, density and energy-weighted density
    // products as split-precision tensor-core GEMMs (`slices` digits of 8 bits); the Cholesky,
    // the reduction to standard form and the eigensolver stay FP64
    int precision = 0;
    int slices = 5;
    // AO count from which the back-transformation of the eigenvectors runs in the compact-WY form
    // (FP64 column strips; with split products the tensor-core GEMM chain) instead of one warp
    // per vector; -1 takes the device's thresholds (tune.h: measured by the autotuner, else the
    // defaults measured once on GB300)
    int blocked_min = -1;
    // back-transformation of n AOs: 0 one warp per vector, 1 FP64 column strips, 2 the
    // split-precision GEMM chain (split mode only, where it beats both FP64 forms)
    int backtransform_form(int n, bool split) const {
        if (blocked_min >= 0) return n >= blocked_min ? (split ? 2 : 1) : 0;
        if (split && n >= tuned_blocked_min(1)) return 2;
        return n >= tuned_blocked_min(0) ? 1 : 0;
    }
    // CUDA stream priority of the single point's stream (lower is more urgent; clamped to the
    // device's range; 0 is the default priority)
    int stream_priority = 0;
    // most blocks of the cooperative tridiagonalisation (0: one per SM); a cap lets concurrent
    // single points share the GPU instead of waiting for all SMs
    int max_coop_blocks = 0;
    // external point charges (xtb_setExternalCharges): charge, position [k][3] (Bohr) and
    // hardness of charge k; empty for none
    std::vector<double> pc_q, pc_xyz, pc_gam;
    // implicit solvent (xtb_setSolvent); solv.on == false for the gas phase
    SolventSpec solv;
};

// Wavefunction kept between calls on the same results object (res%chk of the reference).
struct Wavefunction {
    int nat = 0, nao = 0, nsh = 0;
    std::vector<double> q, qsh, dipm, qp;       // converged (mixed) charges and moments
    std::vector<double> emo, focc;              // orbital energies (Eh) and occupations
    std::vector<double> C;                      // MO coefficients [nao][nao] (row AO, column MO)
    std::vector<double> P;                      // density matrix
    std::vector<double> S;                      // overlap
    bool valid() const { return nat > 0; }
};

struct SPResult {
    double energy = 0.0;
    std::vector<double> gradient;               // [nat][3]
    std::vector<double> dipole;                 // [3]
    std::vector<double> wbo;                    // [nat][nat] Wiberg bond orders (closed shell)
    double hl_gap = 0.0;                        // eV
    int iterations = 0;
    bool converged = false;
    // energy parts (Eh)
    double e_elec = 0, e_rep = 0, e_es = 0, e_aes = 0, e_axc = 0, e_disp = 0, e_atm = 0;
    double gnorm = 0.0;
    double e_pc = 0.0;                          // energy of the shells in the external charges' field
    std::vector<double> pcgrad;                 // [npc][3] gradient on the external charges
    // implicit solvent: free energy of solvation (in the electronic energy) and its parts at the
    // final charges (getEnergyParts, src/solv/gbsa.f90:552-596)
    bool solvated = false;
    double g_solv = 0.0, g_born = 0.0, g_hb = 0.0, g_sasa = 0.0, g_shift = 0.0;
    // device time per phase (ms), measured with CUDA events on the engine stream
    std::vector<double> phase_ms;
    // bytes copied host->device and device->host by this single point
    long long h2d_bytes = 0, d2h_bytes = 0;
    long long launches = 0;   // device kernels launched by this single point
};

// phases timed inside run_singlepoint
enum Phase {
    PH_SETUP = 0,      // uploads, CN, EEQ guess, repulsion
    PH_INTEGRALS,      // S, D, Q, H0 and the Coulomb / AES / D4 kernels
    PH_CHOLESKY,       // S = U^T U, X = U^-1
    PH_HBUILD,         // potentials and H
    PH_STDFORM,        // A = X^T H X (two FP64 GEMMs)
    PH_SYTRD,          // Householder tridiagonalisation
    PH_TRIEIG,         // bisection + inverse iteration (+ cluster re-orthogonalisation)
    PH_BACKTR,         // Q Y and C = X Z
    PH_DENSITY,        // Fermi smearing and P = C f C^T
    PH_POPMIX,         // populations, energies, Broyden
    PH_GRADIENT,       // analytic gradient
    PH_TOTAL,          // whole single point on the device stream
    PH_COUNT
};
extern const char* const kPhaseNames[PH_COUNT];

// Run the single point.  `wfn` is the warm-start wavefunction (used when sizes
// match) and receives the converged one.  Throws std::runtime_error on failure;
// `scc_failed` reports an unconverged SCC (results still filled).  With guess_only the
// call stops after the initial guess and returns it in `wfn` (charges, shell charges,
// zero or warm-start multipoles); `res` is not filled.
void run_singlepoint(const HostMol& hm, const SPSettings& set, Wavefunction& wfn, SPResult& res, bool keep_orbitals,
                     bool& scc_failed, bool guess_only = false);

// Number of CUDA devices visible (0 when none); never throws.
int device_count();

}  // namespace xg
