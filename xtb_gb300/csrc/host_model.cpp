// Host-side molecule set-up for the GFN2 engine (see host_model.h).
//
// Restates newBasisset / slaterToGauss (src/xtb/basisset.f90:33-308, src/slater.f90:373-483),
// initHamiltonian and friends (src/xtb/gfn2.f90:731-967), setzshell / occu
// (src/scc_core.f90:1112-1170, 1509-1542) and newD4Model with the GFN2 reference
// charges (src/disp/dftd4.F90:106-203).
#include "host_model.h"

#include <cmath>
#include <map>
#include <set>

#include "gfn2_params.inc"

namespace xg {

namespace {

constexpr double PI_ = 3.1415926535897932384626433832795029;
const double DFACT[8] = {1.0, 1.0, 3.0, 15.0, 105.0, 945.0, 10395.0, 135135.0};

// Stewart STO-nG expansion with normalisation (src/slater.f90:373-483)
bool slater_to_gauss(int ng, int n, int l, double zeta, double* a, double* c) {
    if ((n > 5 || n <= l) && !(n == 6 && ng == 6)) return false;
    int ityp;
    switch (l) {
        case 0: ityp = n; break;
        case 1: ityp = 4 + n; break;
        case 2: ityp = 7 + n; break;
        case 3: ityp = 9 + n; break;
        default: return false;
    }
    --ityp;
    const double z2 = zeta * zeta;
    for (int k = 0; k < ng; ++k) {
        switch (ng) {
            case 1: a[k] = k_sto_alpha1[ityp] * z2; c[k] = 1.0; break;
            case 2: a[k] = k_sto_alpha2[k][ityp] * z2; c[k] = k_sto_coeff2[k][ityp]; break;
            case 3: a[k] = k_sto_alpha3[k][ityp] * z2; c[k] = k_sto_coeff3[k][ityp]; break;
            case 4: a[k] = k_sto_alpha4[k][ityp] * z2; c[k] = k_sto_coeff4[k][ityp]; break;
            case 5: a[k] = k_sto_alpha5[k][ityp] * z2; c[k] = k_sto_coeff5[k][ityp]; break;
            case 6:
                if (n == 6) {
                    if (l == 0) { a[k] = k_sto_pAlpha6s[k] * z2; c[k] = k_sto_pCoeff6s[k]; }
                    else if (l == 1) { a[k] = k_sto_pAlpha6p[k] * z2; c[k] = k_sto_pCoeff6p[k]; }
                    else return false;
                } else {
                    a[k] = k_sto_alpha6[k][ityp] * z2; c[k] = k_sto_coeff6[k][ityp];
                }
                break;
            default: return false;
        }
    }
    const double top = 2.0 / PI_;
    for (int k = 0; k < ng; ++k)
        c[k] = c[k] * std::pow(top * a[k], 0.75) * std::pow(std::sqrt(4.0 * a[k]), l) / std::sqrt(DFACT[l]);
    return true;
}

int n_primitives(int z, int l, int npq) {
    if (z <= 2) return l == 0 ? 3 : (l == 1 ? 4 : 0);
    switch (l) {
        case 0: case 1: return npq > 5 ? 6 : 4;
        case 2: return 3;
        case 3: return 4;
    }
    return 0;
}

double valence_charge(int z) {
    int core;
    if (z <= 2) core = 0;
    else if (z <= 10) core = 2;
    else if (z <= 18) core = 10;
    else if (z <= 29) core = 18;
    else if (z <= 36) core = 28;
    else if (z <= 47) core = 36;
    else if (z <= 54) core = 46;
    else if (z <= 71) core = 54;
    else if (z <= 79) core = 68;
    else if (z <= 86) core = 78;
    else core = 86;
    double v = z - core;
    if (z > 57 && z < 72) v = 3.0;
    return v;
}

double zeta_fn(double a, double c, double qref, double qmod) {
    if (qmod < 0.0) return std::exp(a);
    return std::exp(a * (1.0 - std::exp(c * (1.0 - qref / qmod))));
}

// trapezoidal Casimir-Polder integration weights (trapzd, src/disp/dftd4.F90:381-449)
void trap_weights(double* w) {
    const double f[23] = {0.000001, 0.05, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0,
                          1.2, 1.4, 1.6, 1.8, 2.0, 2.5, 3.0, 4.0, 5.0, 7.5, 10.0};
    w[0] = 0.5 * (f[1] - f[0]);
    for (int k = 1; k < 22; ++k) w[k] = 0.5 * ((f[k] - f[k - 1]) + (f[k + 1] - f[k]));
    w[22] = 0.5 * (f[22] - f[21]);
}

}  // namespace

double chemical_hardness(int Z) { return (Z >= 1 && Z <= 86) ? k_chemicalHardness[Z - 1] : 0.0; }

std::string build_host_mol(int nat, const int* Zin, const double* xyzin, double charge, int uhf, HostMol& hm) {
    hm = HostMol();
    if (nat <= 0) return "molecule has no atoms";
    hm.nat = nat;
    hm.charge = charge;
    hm.uhf = uhf;
    hm.Z.assign(Zin, Zin + nat);
    hm.xyz.assign(xyzin, xyzin + 3 * nat);
    std::map<int, int> elem;
    for (int i = 0; i < nat; ++i) {
        const int z = hm.Z[i];
        if (z < 1 || z > 86) return "element Z=" + std::to_string(z) + " is not parametrised in GFN2-xTB";
        if (!elem.count(z)) {
            const int id = (int)elem.size();
            elem[z] = id;
            hm.elem_Z.push_back(z);
        }
    }
    hm.nelem = (int)elem.size();
    // every later stage divides by interatomic distances: reject non-finite coordinates and
    // atoms that sit on top of each other (closer than 1e-3 bohr) before any device work
    for (int i = 0; i < 3 * nat; ++i)
        if (!std::isfinite(hm.xyz[i])) return "atom " + std::to_string(i / 3 + 1) + " has a non-finite coordinate";
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < i; ++j) {
            const double dx = hm.xyz[3 * i] - hm.xyz[3 * j], dy = hm.xyz[3 * i + 1] - hm.xyz[3 * j + 1],
                         dz = hm.xyz[3 * i + 2] - hm.xyz[3 * j + 2];
            if (dx * dx + dy * dy + dz * dz < 1e-6)
                return "atoms " + std::to_string(j + 1) + " and " + std::to_string(i + 1) + " coincide";
        }
    // per-atom data
    double zsum = 0.0;
    for (int i = 0; i < nat; ++i) {
        const int z = hm.Z[i], iz = z - 1;
        hm.eid.push_back(elem[z]);
        hm.zval.push_back(valence_charge(z));
        zsum += hm.zval.back();
        hm.rcov.push_back(k_covalentRadD3[iz]);
        hm.en.push_back(k_paulingEN[iz]);
        hm.rcov4.push_back(k_rcovD4[iz]);
        hm.en4.push_back(k_enD4[iz]);
        hm.eeq_en.push_back(k_eeq_en[iz]);
        hm.eeq_gam.push_back(k_eeq_gam[iz]);
        hm.eeq_kappa.push_back(k_eeq_kappa[iz]);
        hm.eeq_alpha.push_back(k_eeq_alpha[iz]);
        hm.mrad.push_back(k_multiRad[iz]);
        hm.valcn.push_back(k_valenceCN[iz]);
        hm.dkern.push_back(k_dipKernel[iz]);
        hm.qkern.push_back(k_quadKernel[iz]);
        hm.rep_alpha.push_back(k_repAlpha[iz]);
        hm.rep_zeff.push_back(k_repZeff[iz]);
        hm.r4r2.push_back(k_sqrtZr4r2[iz]);
        hm.arad.push_back(k_atomicRad[iz]);
    }
    // electrons and occupations (occu, src/scc_core.f90:1112-1170)
    hm.nel = (int)std::lround(zsum - charge);
    int nopen = uhf;
    if (nopen == 0 && hm.nel % 2 != 0) nopen = 1;
    // basis
    int ao = 0;
    for (int i = 0; i < nat; ++i) {
        const int z = hm.Z[i], iz = z - 1;
        hm.at_sh0.push_back((int)hm.sh_atom.size());
        hm.at_ao0.push_back(ao);
        const int nsh = k_nShell[iz];
        hm.at_nsh.push_back(nsh);
        bool seen[4] = {false, false, false, false};
        double ntot = -1.0e-6;
        for (int s = 0; s < nsh; ++s) {
            const int l = k_angShell[s][iz];
            const int npq = k_principalQuantumNumber[s][iz];
            if (l > 2) return "f shells are not supported";
            if (seen[l]) return "non-valence shells do not occur in GFN2-xTB";
            seen[l] = true;
            const int ng = n_primitives(z, l, npq);
            double a[HMAXPRIM] = {0}, c[HMAXPRIM] = {0};
            const double zeta = k_slaterExponent[s][iz];
            if (!slater_to_gauss(ng, npq, l, zeta, a, c)) return "STO-nG expansion failed for Z=" + std::to_string(z);
            hm.sh_atom.push_back(i);
            hm.sh_l.push_back(l);
            hm.sh_ao.push_back(ao);
            hm.sh_nprim.push_back(ng);
            for (int k = 0; k < HMAXPRIM; ++k) {
                hm.sh_alpha.push_back(k < ng ? a[k] : 1.0);
                hm.sh_coef.push_back(k < ng ? c[k] : 0.0);
            }
            hm.sh_zeta.push_back(zeta);
            hm.sh_se0.push_back(k_selfEnergy[s][iz]);
            hm.sh_kcn.push_back(k_kCNL[l][iz]);
            hm.sh_poly.push_back(k_shellPolyL[l][iz]);
            hm.sh_eta.push_back(k_chemicalHardness[iz] * (1.0 + k_shellHardness[l][iz]));
            const int kind = k_gfn2Kinds[iz];
            const double gam3 = (l == 0) ? 1.0 : (l == 1 ? 0.5 : 0.25);
            (void)kind;  // both kinds share the same gam3shell table in GFN2
            hm.sh_gam3.push_back(k_thirdOrderAtom[iz] * gam3);
            const double refocc = k_referenceOccL[l][iz];
            hm.sh_refocc.push_back(refocc);
            double zs = refocc;
            ntot += zs;
            if (ntot > hm.zval[i]) zs = 0.0;
            hm.sh_zsh.push_back(zs);
            for (int k = 0; k < 2 * l + 1; ++k) {
                hm.ao_sh.push_back((int)hm.sh_atom.size() - 1);
                hm.ao_at.push_back(i);
            }
            ao += 2 * l + 1;
        }
        hm.at_nao.push_back(ao - hm.at_ao0.back());
    }
    hm.nsh = (int)hm.sh_atom.size();
    hm.nao = ao;
    hm.sh_byl.clear();
    for (int l = 0; l < 3; ++l) {
        hm.l_off[l] = (int)hm.sh_byl.size();
        for (int s = 0; s < hm.nsh; ++s)
            if (hm.sh_l[s] == l) hm.sh_byl.push_back(s);
    }
    hm.l_off[3] = (int)hm.sh_byl.size();
    if (hm.nel < 0) return "negative number of electrons";
    if (hm.nel > 2 * hm.nao) return "Not enough basis functions for filling orbitals";
    {
        // occu: integer occupations -> number of alpha / beta electrons
        std::vector<int> focc(hm.nao, 0);
        if (hm.nel % 2 == 0) {
            int ihomo = hm.nel / 2;
            for (int i = 0; i < ihomo; ++i) focc[i] = 2;
            if (2 * ihomo != hm.nel) { ++ihomo; focc[ihomo - 1] = 1; if (nopen == 0) nopen = 1; }
            if (nopen > 1)
                for (int i = 1; i <= nopen / 2; ++i) { focc[ihomo - i] -= 1; focc[ihomo + i - 1] += 1; }
        } else {
            const int na = hm.nel / 2 + (nopen - 1) / 2 + 1;
            const int nb = hm.nel / 2 - (nopen - 1) / 2;
            for (int i = 0; i < na && i < hm.nao; ++i) focc[i] += 1;
            for (int i = 0; i < nb && i < hm.nao; ++i) focc[i] += 1;
        }
        int ia = 0, ib = 0;
        for (int i = 0; i < hm.nao; ++i) {
            if (focc[i] >= 1) ia = i + 1;
            if (focc[i] == 2) ib = i + 1;
        }
        hm.nel_a = ia;
        hm.nel_b = ib;
    }
    // D4 model for the elements present (newD4Model with p_refq_gfn2xtb: secq = 0)
    const int ne = hm.nelem;
    hm.d4_nref.assign(ne, 0);
    hm.d4_ncount.assign(ne * HMAXREF, 0);
    hm.d4_zeff.assign(ne, 0.0);
    hm.d4_gam.assign(ne, 0.0);
    hm.d4_refq.assign(ne * HMAXREF, 0.0);
    hm.d4_refcn.assign(ne * HMAXREF, 0.0);
    std::vector<double> alpha((size_t)ne * HMAXREF * 23, 0.0);
    for (int e = 0; e < ne; ++e) {
        const int z = hm.elem_Z[e], iz = z - 1;
        const int nref = k_d4_refn[iz];
        hm.d4_nref[e] = nref;
        hm.d4_zeff[e] = k_d4_zeff[iz];
        hm.d4_gam[e] = k_d4_gam[iz];
        int cncount[19] = {0};
        cncount[0] = 1;
        for (int r = 0; r < nref; ++r) {
            const int is = k_d4_refsys[r][iz];
            const double izf = k_d4_zeff[is - 1];
            const double zf = zeta_fn(3.0, k_d4_gam[is - 1] * 2.0, 0.0 + izf, k_d4_refh[r][iz] + izf);
            for (int f = 0; f < 23; ++f) {
                const double sec = k_d4_sscale[is - 1] * k_d4_secaiw[f][is - 1] * zf;
                const double v = k_d4_ascale[r][iz] * (k_d4_alphaiw[f][r][iz] - k_d4_hcount[r][iz] * sec);
                alpha[((size_t)e * HMAXREF + r) * 23 + f] = v > 0.0 ? v : 0.0;
            }
            const int icn = (int)std::lround(k_d4_refcn[r][iz]);
            cncount[icn] += 1;
            hm.d4_refq[e * HMAXREF + r] = k_d4_refq[r][iz];
            hm.d4_refcn[e * HMAXREF + r] = k_d4_refcovcn[r][iz];
        }
        for (int r = 0; r < nref; ++r) {
            const int c = cncount[(int)std::lround(k_d4_refcn[r][iz])];
            hm.d4_ncount[e * HMAXREF + r] = c * (c + 1) / 2;
        }
    }
    double w[23];
    trap_weights(w);
    const double thopi = 3.0 / PI_;
    hm.d4_c6.assign((size_t)ne * ne * HMAXREF * HMAXREF, 0.0);
    for (int e1 = 0; e1 < ne; ++e1)
        for (int e2 = 0; e2 < ne; ++e2)
            for (int r = 0; r < hm.d4_nref[e1]; ++r)
                for (int s = 0; s < hm.d4_nref[e2]; ++s) {
                    double sum = 0.0;
                    for (int f = 0; f < 23; ++f)
                        sum += alpha[((size_t)e1 * HMAXREF + r) * 23 + f] * alpha[((size_t)e2 * HMAXREF + s) * 23 + f] * w[f];
                    hm.d4_c6[(((size_t)e1 * ne + e2) * HMAXREF + r) * HMAXREF + s] = thopi * sum;
                }
    return "";
}

void ini_qshell(const HostMol& hm, const double* q, double* qsh) {
    for (int i = 0; i < hm.nat; ++i) {
        double ntot = -1.0e-6;
        for (int s = hm.at_sh0[i]; s < hm.at_sh0[i] + hm.at_nsh[i]; ++s) {
            double zs = hm.sh_refocc[s];
            ntot += zs;
            if (ntot > hm.zval[i]) zs = 0.0;
            qsh[s] = zs / hm.zval[i] * q[i];
        }
    }
}

}  // namespace xg
