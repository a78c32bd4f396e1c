// GBSA / ALPB implicit solvation for the plain single point (TBorn of src/solv/gbsa.f90).
//
// Host side: xtb_setSolvent's choice resolved against the GFN2 parameter tables, and the
// per-molecule model (radii, surface tensions, H-bond strengths, Lebedev grid, SASA neighbour
// lists).  Device side: Born radii (GBOBC-II), the numerical solvent-accessible surface, the
// Born matrix B (Still, P16 or salt-screened Still kernel, H-bond diagonal, ALPB shape term),
// the SCC potential B q and energy 1/2 q^T B q + G_sasa + G_shift, and the analytic gradient.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace xg {

// the solvation input of a calculator (TSolvInput, src/solv/input.F90, as xtb_setSolvent fills it)
struct SolventSpec {
    bool on = false;
    std::string solvent;          // normalised solvent name
    int kernel = 0;               // 0: Still kernel with the GBSA parameter sets, 1: P16 with the ALPB sets
    bool alpb = false;            // ALPB shape correction
    int state = 1;                // solution state: 1 gsolv, 2 reference (1 M gas / 1 M solution), 3 1 bar
    double temperature = 298.15;  // K
    int nang = 230;               // requested angular grid points per atom
    double ion_strength = 0.0;    // salt (mol/L); > 0 selects the Debye-Hueckel screened Still kernel
    double ion_rad = 0.0;         // ion radius (Bohr)
    int set = -1;                 // index of the parameter set
};

// Resolve (solvent, model) to a spec: model "gbsa" or "alpb"; the other models of the reference
// ("cosmo", "tmcosmo", "cpcmx") are refused.  Returns "" on success, else the error message.
// A solvent "none", "gas" or "vac" gives a spec with on == false (no solvation).
// `kernel` (-1: the model's own) replaces the kernel and with it the parameter sets, as
// TSolvInput%kernel does (the reference's tests pair the ALPB correction with the Still kernel).
std::string make_solvent_spec(const std::string& solvent, const std::string& model, int state, double temperature,
                              int nang, SolventSpec& out, int kernel = -1);

// The per-molecule model (initBorn, src/solv/gbsa.f90:217-389)
struct SolvHost {
    int nat = 0, npt = 0;
    int kernel = 0;
    bool alpb = false, lhb = false, lsalt = false;
    double eps = 0.0, keps = 0.0, alpbet = 0.0, c1 = 0.0, gshift = 0.0, srcut = 0.0, kappa = 0.0, ion_rad = 0.0;
    // per atom: van der Waals radius, descreening radius rho, offset radius svdw, SASA radius,
    // SASA weight prefactor wrp, surface tension, H-bond strength
    std::vector<double> vdwr, rho, svdw, vdwsa, wrp, gamsasa, hbmag;
    std::vector<double> grid;     // [npt][4]: unit vector and weight
    std::vector<int> nb_off, nb;  // neighbours closer than srcut (CSR, increasing index)
};
// `xyz` [nat][3] in Bohr (the SASA neighbour lists depend on the geometry)
void build_solv_host(const SolventSpec& spec, int nat, const int* Z, const double* xyz, SolvHost& out);

// device buffers of one single point (carved from the engine's workspace)
struct SolvDev {
    int nat = 0, npt = 0, kernel = 0;
    bool alpb = false, lhb = false, lsalt = false;
    double keps = 0.0, alpbet = 0.0, c1 = 0.0, gshift = 0.0, eps = 0.0, kappa = 0.0, ion_rad = 0.0;
    const double *vdwr, *rho, *svdw, *vdwsa, *wrp, *gamsasa, *hbmag, *grid;
    const int *nb_off, *nb;
    double *brad, *dbrad, *sasa, *sasap, *B, *hbw, *ionscr, *discr, *aux, *bq, *grddb, *wsur, *esolv;
};
// geometry-dependent set-up: Born radii, SASA, H-bond weights, ALPB shape, Born matrix
void solv_update(cudaStream_t st, const SolvDev& s, const double* xyz);
// atomic potential: vat += B q
void solv_shift(cudaStream_t st, const SolvDev& s, const double* q, double* vat);
// esolv[0] = 1/2 q^T B q + G_sasa + G_shift; esolv[1] = G_hb; esolv[2] = G_sasa; esolv[3] = G_shift
void solv_energy(cudaStream_t st, const SolvDev& s, const double* q);
// grad += dG_solv/dR at the charges q
void solv_gradient(cudaStream_t st, const SolvDev& s, const double* xyz, const double* q, double* grad);

}  // namespace xg
