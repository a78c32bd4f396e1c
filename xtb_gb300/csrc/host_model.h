// Host-side set-up of one molecule for the GFN2 engine: parameters per atom and
// shell, the contracted STO-nG basis, and the D4 reference C6 tables of the
// elements present.  O(N) work, done once per molecule on the CPU.
#pragma once
#include <string>
#include <vector>

namespace xg {

constexpr int HMAXPRIM = 6;
constexpr int HMAXREF = 7;

struct HostMol {
    int nat = 0, nsh = 0, nao = 0, nelem = 0;
    double charge = 0.0;
    int uhf = 0;
    int nel = 0;             // number of electrons
    int nel_a = 0, nel_b = 0;// alpha / beta electrons (occu)
    std::vector<int> Z, eid, at_sh0, at_nsh, at_ao0, at_nao;
    std::vector<double> xyz;
    std::vector<double> zval;   // valence charge
    std::vector<double> rcov, en, rcov4, en4, eeq_en, eeq_gam, eeq_kappa, eeq_alpha, mrad, valcn, dkern, qkern,
        rep_alpha, rep_zeff, r4r2, arad;
    // elements
    std::vector<int> elem_Z, d4_nref, d4_ncount;
    std::vector<double> d4_zeff, d4_gam, d4_refq, d4_refcn, d4_c6;
    // shells
    std::vector<int> sh_atom, sh_l, sh_ao, sh_nprim;
    std::vector<double> sh_alpha, sh_coef, sh_zeta, sh_se0, sh_kcn, sh_poly, sh_eta, sh_gam3, sh_zsh, sh_refocc;
    // AOs
    std::vector<int> ao_sh, ao_at;
    // shells grouped by angular momentum (increasing index within a group): group l is
    // sh_byl[l_off[l] .. l_off[l + 1])
    std::vector<int> sh_byl;
    int l_off[4] = {0, 0, 0, 0};
};

// Returns an empty string on success, else an error message (unsupported element, ...).
std::string build_host_mol(int nat, const int* Z, const double* xyz, double charge, int uhf, HostMol& hm);
// GFN2-xTB chemical hardness of element Z (1..86; 0 outside), the hardness an external point
// charge of that element takes (setExternalCharges_api, src/api/calculator.f90:482-537)
double chemical_hardness(int Z);
// iniqshell (src/scc_core.f90:1475-1506): shell charges from atomic charges
void ini_qshell(const HostMol& hm, const double* q, double* qsh);

}  // namespace xg
