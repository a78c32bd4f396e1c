// C ABI of the GB300 GFN2-xTB engine: drop-in for the reference xtb C API.
//
// Handle life cycle, error log and argument checks restate the reference's
// bind(C) layer (src/api/environment.f90:47-245, src/api/molecule.f90:47-137,
// src/api/calculator.f90:58-699, src/api/interface.f90:40-156,
// src/api/results.f90:54-504).  Unlike the reference, no state is global: every
// handle owns its data, so different threads may drive different handles
// concurrently; the device work of one call is serialised on the calling
// thread's CUDA stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/xtb_gb300.h"
#include "batch.h"
#include "engine.h"
#include "tune.h"
#include "serve.h"
#include "splitgemm.h"
#include "host_model.h"
#include "linalg.h"

struct LogEntry {
    bool error;
    std::string text;
};

struct _xtb_TEnvironment {
    std::vector<LogEntry> log;
    int verbosity = XTB_VERBOSITY_FULL;
    FILE* out = stdout;
    bool own_out = false;
    void error(const std::string& msg, const char* source) { log.push_back({true, std::string(source) + ": " + msg}); }
    void warning(const std::string& msg, const char* source) { log.push_back({false, std::string(source) + ": " + msg}); }
    bool failed() const {
        for (auto& e : log)
            if (e.error) return true;
        return false;
    }
};

struct _xtb_TMolecule {
    int nat = 0;
    std::vector<int> Z;
    std::vector<double> xyz;
    double charge = 0.0;
    int uhf = 0;
};

struct _xtb_TCalculator {
    bool loaded = false;
    bool keep_orbitals = true;
    xg::SPSettings set;
    int nat = 0;
    std::vector<int> Z;   // element list the parametrisation was loaded for
};

struct _xtb_TResults {
    bool has = false;
    xg::Wavefunction wfn;
    xg::SPResult sp;
    int nat = 0;
    std::vector<double> xyz;   // geometry of the last single point (virial)
};

namespace {

constexpr int kMaxElem = 86;   // GFN2-xTB parametrisation (src/xtb/gfn2.f90:70)

bool check_env(xtb_TEnvironment env) { return env != nullptr; }

}  // namespace

extern "C" {

int xtb_getAPIVersion(void) { return XTB_API_VERSION; }

// ------------------------------------------------------------------ environment
xtb_TEnvironment xtb_newEnvironment(void) { return new _xtb_TEnvironment(); }

void xtb_delEnvironment(xtb_TEnvironment* env) {
    if (env && *env) {
        if ((*env)->own_out && (*env)->out) fclose((*env)->out);
        delete *env;
        *env = nullptr;
    }
}

int xtb_checkEnvironment(xtb_TEnvironment env) {
    if (!check_env(env)) return 0;
    return env->failed() ? 1 : 0;
}

void xtb_showEnvironment(xtb_TEnvironment env, const char* message) {
    if (!check_env(env) || env->log.empty()) return;
    FILE* f = env->out ? env->out : stdout;
    fprintf(f, "########################################################################\n");
    fprintf(f, "[%s] %s\n", env->failed() ? "ERROR" : "WARNING", message ? message : "");
    for (size_t i = env->log.size(); i-- > 0;) fprintf(f, "-%zu- %s\n", i + 1, env->log[i].text.c_str());
    fprintf(f, "########################################################################\n");
    fflush(f);
    env->log.clear();
}

void xtb_getError(xtb_TEnvironment env, char* buffer, const int* buffersize) {
    if (!check_env(env) || !buffer) return;
    if (!env->failed()) return;
    std::string msg;
    for (size_t i = env->log.size(); i-- > 0;) {
        if (!msg.empty()) msg += "\n";
        msg += "-" + std::to_string(i + 1) + "- " + env->log[i].text;
    }
    env->log.clear();
    const size_t cap = buffersize ? (size_t)std::max(*buffersize, 0) : msg.size() + 1;
    if (cap == 0) return;
    const size_t n = std::min(msg.size(), cap - 1);
    memcpy(buffer, msg.data(), n);
    buffer[n] = '\0';
}

void xtb_setOutput(xtb_TEnvironment env, const char* filename) {
    xtb_releaseOutput(env);
    if (!check_env(env) || !filename) return;
    const std::string f(filename);
    if (f == "-" || f == "STDOUT") env->out = stdout;
    else if (f == "STDERR") env->out = stderr;
    else {
        FILE* fp = fopen(filename, "w");
        if (!fp) {
            env->error("cannot open output file " + f, "xtb_api_setOutput");
            return;
        }
        env->out = fp;
        env->own_out = true;
    }
}

void xtb_releaseOutput(xtb_TEnvironment env) {
    if (!check_env(env)) return;
    if (env->own_out && env->out) fclose(env->out);
    env->own_out = false;
    env->out = stdout;
}

void xtb_setVerbosity(xtb_TEnvironment env, int verbosity) {
    if (!check_env(env)) return;
    if (verbosity < 0 || verbosity > 2) env->warning("Verbosity specified is out of range", "xtb_api_setVerbosity");
    env->verbosity = verbosity;
}

// ------------------------------------------------------------------ molecule
xtb_TMolecule xtb_newMolecule(xtb_TEnvironment env, const int* natoms, const int* numbers, const double* positions,
                              const double* charge, const int* uhf, const double* lattice, const bool* periodic) {
    const char* src = "xtb_api_newMolecule";
    if (!check_env(env)) return nullptr;
    if (!natoms || *natoms <= 0) {
        env->error("Number of atoms must be positive", src);
        return nullptr;
    }
    const int n = *natoms;
    if (!numbers || !positions) {
        env->error("Could not generate molecular structure", src);
        return nullptr;
    }
    for (int i = 0; i < n; ++i)
        if (numbers[i] <= 0 || numbers[i] > 118) {
            env->error("Invalid atomic number present", src);
            return nullptr;
        }
    if (periodic && (periodic[0] || periodic[1] || periodic[2])) {
        env->error("Periodic boundary conditions are not supported by this engine", src);
        return nullptr;
    }
    (void)lattice;
    for (int i = 0; i < 3 * n; ++i)
        if (!std::isfinite(positions[i])) {
            env->error("Could not generate molecular structure", src);
            return nullptr;
        }
    auto* mol = new _xtb_TMolecule();
    mol->nat = n;
    mol->Z.assign(numbers, numbers + n);
    mol->xyz.assign(positions, positions + 3 * n);
    mol->charge = charge ? *charge : 0.0;
    mol->uhf = uhf ? *uhf : 0;
    return mol;
}

void xtb_delMolecule(xtb_TMolecule* mol) {
    if (mol && *mol) {
        delete *mol;
        *mol = nullptr;
    }
}

void xtb_updateMolecule(xtb_TEnvironment env, xtb_TMolecule mol, const double* positions, const double* lattice) {
    const char* src = "xtb_api_updateMolecule";
    if (!check_env(env)) return;
    if (!mol) {
        env->error("Molecular structure data is not allocated", src);
        return;
    }
    if (!positions) {
        env->error("Position array is not allocated", src);
        return;
    }
    (void)lattice;
    mol->xyz.assign(positions, positions + 3 * mol->nat);
}

// ------------------------------------------------------------------ calculator
xtb_TCalculator xtb_newCalculator(void) { return new _xtb_TCalculator(); }

void xtb_delCalculator(xtb_TCalculator* calc) {
    if (calc && *calc) {
        delete *calc;
        *calc = nullptr;
    }
}

void xtb_loadGFN2xTB(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, char* filename) {
    const char* src = "xtb_api_loadGFN2xTB";
    if (!check_env(env)) return;
    if (!mol) {
        env->error("Molecular structure data is not allocated", src);
        return;
    }
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", src);
        return;
    }
    (void)filename;   // the GFN2-xTB parameter set is built in
    for (int z : mol->Z)
        if (z > kMaxElem) {
            env->error("Element not parametrised for GFN2-xTB", src);
            return;
        }
    calc->loaded = true;
    calc->nat = mol->nat;
    calc->Z = mol->Z;
}

static void unsupported(xtb_TEnvironment env, const char* what, const char* src) {
    if (check_env(env)) env->error(std::string(what) + " is not supported by the GB300 GFN2-xTB engine", src);
}

void xtb_loadGFN0xTB(xtb_TEnvironment env, xtb_TMolecule, xtb_TCalculator, char*) {
    unsupported(env, "GFN0-xTB", "xtb_api_loadGFN0xTB");
}
void xtb_loadGFN1xTB(xtb_TEnvironment env, xtb_TMolecule, xtb_TCalculator, char*) {
    unsupported(env, "GFN1-xTB", "xtb_api_loadGFN1xTB");
}
void xtb_loadGFNFF(xtb_TEnvironment env, xtb_TMolecule, xtb_TCalculator, char*) {
    unsupported(env, "GFN-FF", "xtb_api_loadGFNFF");
}
// implicit solvent (setSolvent_api, src/api/calculator.f90:341-439): state, temperature, grid and
// model are optional (NULL: gsolv, 298.15 K, 230 points, "gbsa")
void xtb_setSolvent(xtb_TEnvironment env, xtb_TCalculator calc, char* solvent, int* state, double* temperature,
                    int* grid, char* model) {
    static const char* src = "xtb_api_setSolvent";
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", src);
        return;
    }
    if (!calc->loaded) {
        env->error("No calculator loaded to add solvation model", src);
        return;
    }
    if (!solvent) {
        env->error("Solvent name is missing", src);
        return;
    }
    xg::SolventSpec spec;
    const std::string err = xg::make_solvent_spec(solvent, model ? model : "gbsa", state ? *state : 1,
                                                  temperature ? *temperature : 298.15, grid ? *grid : 230, spec);
    if (!err.empty()) {
        env->error(err, err == "Unknown solvation model" ? src : "solv_model_loadInternalParam");
        if (err != "Unknown solvation model")
            env->error(std::string("Could not add solvation model for '") + solvent + "'", src);
        return;
    }
    spec.ion_strength = calc->set.solv.ion_strength;   // salt set through xtbgb_setSolventSalt is kept
    spec.ion_rad = calc->set.solv.ion_rad;
    calc->set.solv = spec;
}

void xtb_releaseSolvent(xtb_TEnvironment env, xtb_TCalculator calc) {
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", "xtb_api_setRelease");
        return;
    }
    calc->set.solv = xg::SolventSpec();
}
namespace {
// external point charges on a loaded calculator (setExternalCharges_api,
// src/api/calculator.f90:482-537); gam null: the hardness of each charge's element
void set_external_charges(xtb_TEnvironment env, xtb_TCalculator calc, int npc, const int* numbers,
                          const double* charges, const double* positions, const double* gam, const char* src) {
    if (npc <= 0) {
        env->error("Negative number of point charges provided", src);
        return;
    }
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", src);
        return;
    }
    if (!calc->loaded) {
        env->error("No calculator loaded to add external potential", src);
        return;
    }
    if (!charges || !positions || (!gam && !numbers)) {
        env->error("External charges, positions or numbers are missing", src);
        return;
    }
    std::vector<double> q(charges, charges + npc), x(positions, positions + 3 * (size_t)npc), g(npc);
    for (int k = 0; k < npc; ++k) {
        if (gam) {
            g[k] = gam[k];
        } else {
            if (numbers[k] < 1 || numbers[k] > kMaxElem) {
                env->error("Invalid element for an external charge: " + std::to_string(numbers[k]), src);
                return;
            }
            g[k] = xg::chemical_hardness(numbers[k]);
        }
        if (!(g[k] > 0.0) || !std::isfinite(q[k]) || !std::isfinite(x[3 * k]) || !std::isfinite(x[3 * k + 1]) ||
            !std::isfinite(x[3 * k + 2])) {
            env->error("External charge " + std::to_string(k + 1) + " has an invalid charge, position or hardness",
                       src);
            return;
        }
    }
    calc->set.pc_q = std::move(q);
    calc->set.pc_xyz = std::move(x);
    calc->set.pc_gam = std::move(g);
}
}  // namespace

void xtb_setExternalCharges(xtb_TEnvironment env, xtb_TCalculator calc, int* n, int* numbers, double* charges,
                            double* positions) {
    if (!check_env(env)) return;
    set_external_charges(env, calc, n ? *n : 0, numbers, charges, positions, nullptr, "xtb_api_setExternalCharges");
}

void xtb_releaseExternalCharges(xtb_TEnvironment env, xtb_TCalculator calc) {
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", "xtb_api_releaseExternalCharges");
        return;
    }
    calc->set.pc_q.clear();
    calc->set.pc_xyz.clear();
    calc->set.pc_gam.clear();
}

void xtb_setAccuracy(xtb_TEnvironment env, xtb_TCalculator calc, double accuracy) {
    const char* src = "xtb_api_setAccuracy";
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", src);
        return;
    }
    if (!calc->loaded) {
        env->error("Setting accuracy not possible, no calculator loaded", src);
        return;
    }
    if (accuracy < 1.0e-4) {
        env->warning("We cannot provide this level of accuracy, resetted accuracy to 0.0001", src);
        accuracy = 1.0e-4;
    } else if (accuracy > 1.0e3) {
        env->warning("We cannot provide this level of accuracy, resetted accuracy to 1000", src);
        accuracy = 1.0e3;
    }
    calc->set.accuracy = accuracy;
}

void xtb_setMaxIter(xtb_TEnvironment env, xtb_TCalculator calc, int iterations) {
    const char* src = "xtb_api_setMaxIter";
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", src);
        return;
    }
    if (!calc->loaded) {
        env->error("Setting iterations not possible, no calculator loaded", src);
        return;
    }
    calc->set.maxiter = std::max(iterations, 1);
}

void xtb_setElectronicTemp(xtb_TEnvironment env, xtb_TCalculator calc, double temperature) {
    const char* src = "xtb_api_setElectronicTemp";
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", src);
        return;
    }
    if (!calc->loaded) {
        env->error("Setting electronic temperature not possible, no calculator loaded", src);
        return;
    }
    calc->set.etemp = std::max(temperature, 1.0e-6);
}

// ------------------------------------------------------------------ single point
void xtb_singlepoint(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, xtb_TResults res) {
    const char* src = "xtb_api_singlepoint";
    if (!check_env(env)) return;
    if (!mol) {
        env->error("Molecular structure data is not allocated", src);
        return;
    }
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", src);
        return;
    }
    if (!calc->loaded) {
        env->error("No calculator loaded for single point", src);
        return;
    }
    if (!res) {
        env->error("Calculation results are not allocated", src);
        return;
    }
    xg::HostMol hm;
    const std::string err = xg::build_host_mol(mol->nat, mol->Z.data(), mol->xyz.data(), mol->charge, mol->uhf, hm);
    if (!err.empty()) {
        env->error(err, "xtb_calculator_singlepoint");
        env->error("Electronic structure method terminated", "xtb_calculator_singlepoint");
        return;
    }
    // warm start only when the sizes of the kept wavefunction match (src/api/interface.f90:83-92)
    if (res->wfn.valid() && (res->wfn.nat != hm.nat || res->wfn.nao != hm.nao || res->wfn.nsh != hm.nsh))
        res->wfn = xg::Wavefunction();
    bool failed = false;
    try {
        xg::run_singlepoint(hm, calc->set, res->wfn, res->sp, calc->keep_orbitals, failed);
    } catch (const std::exception& e) {
        env->error(e.what(), "scf");
        env->error("Electronic structure method terminated", "xtb_calculator_singlepoint");
        res->has = false;
        return;
    }
    res->has = true;
    res->nat = hm.nat;
    res->xyz = mol->xyz;
    if (failed) env->error("Self consistent charge iterator did not converge", "scf");
    if (env->verbosity >= XTB_VERBOSITY_MINIMAL && env->out) {
        fprintf(env->out, "          | TOTAL ENERGY %28.12f Eh   |\n", res->sp.energy);
        fprintf(env->out, "          | GRADIENT NORM %27.12f Eh/a0|\n", res->sp.gnorm);
        fprintf(env->out, "          | HOMO-LUMO GAP %27.12f eV   |\n", res->sp.hl_gap);
        fflush(env->out);
    }
}

// ------------------------------------------------------------------ Hessian
void xtb_hessian(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, xtb_TResults res, double* hessian,
                 int* atom_index_list, int* step_size, double* dipole_gradient, double* polarizability_gradient) {
    static const char* src = "xtb_api_hessian";
    if (!check_env(env)) return;
    if (!mol) {
        env->error("Molecular structure data is not allocated", src);
        return;
    }
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", src);
        return;
    }
    if (!calc->loaded) {
        env->error("No calculator loaded for single point", src);
        return;
    }
    if (!res) {
        env->error("Calculation results are not allocated", src);
        return;
    }
    if (!hessian) {
        env->error("Hessian array is not allocated", src);
        return;
    }
    if (atom_index_list || step_size) {
        env->error("Atom lists and step sizes are not supported: pass NULL (all atoms, step 0.005 Bohr)", src);
        return;
    }
    if (polarizability_gradient) {
        env->error("Polarizability gradients are not available for GFN2-xTB here", src);
        return;
    }
    const int n = mol->nat;
    xg::HostMol hm0;
    std::string err = xg::build_host_mol(n, mol->Z.data(), mol->xyz.data(), mol->charge, mol->uhf, hm0);
    if (!err.empty()) {
        env->error(err, src);
        return;
    }
    const double step = 0.005, step2 = 0.5 / step;
    try {
        // every displaced point starts from the results object's wavefunction; a fresh object gets
        // the initial guess of the undisplaced molecule (hessian_api, src/api/interface.f90:374-391)
        if (!(res->wfn.valid() && res->wfn.nat == hm0.nat && res->wfn.nao == hm0.nao && res->wfn.nsh == hm0.nsh)) {
            xg::Wavefunction g;
            xg::SPResult dummy;
            bool failed = false;
            xg::run_singlepoint(hm0, calc->set, g, dummy, false, failed, true);
            res->wfn = g;
        }
        const xg::Wavefunction* chk0 = &res->wfn;
        std::vector<xg::HostMol> mols(6 * (size_t)n);
        std::vector<const xg::Wavefunction*> guesses(mols.size(), chk0);
        for (int iat = 0; iat < n; ++iat)
            for (int ic = 0; ic < 3; ++ic)
                for (int sg = 0; sg < 2; ++sg) {
                    std::vector<double> xyz = mol->xyz;
                    xyz[3 * iat + ic] += sg == 0 ? step : -step;
                    err = xg::build_host_mol(n, mol->Z.data(), xyz.data(), mol->charge, mol->uhf,
                                             mols[2 * (3 * iat + ic) + sg]);
                    if (!err.empty()) throw std::runtime_error(err);
                }
        xg::BatchSettings set;
        set.accuracy = calc->set.accuracy;
        set.etemp = calc->set.etemp;
        set.maxiter = calc->set.maxiter;
        xg::BatchResults br;
        if (calc->set.solv.on || !calc->set.pc_q.empty()) {
            // an implicit solvent or external charges: the displaced points run on the plain
            // engine, which carries both (the batched engine is gas phase only)
            const size_t nm = mols.size();
            br.status.assign(nm, xg::BST_OK);
            br.gradient.assign(3 * (size_t)n * nm, 0.0);
            br.dipole.assign(3 * nm, 0.0);
            for (size_t k = 0; k < nm; ++k) {
                xg::Wavefunction w = *chk0;
                xg::SPResult r;
                bool failed = false;
                xg::run_singlepoint(mols[k], calc->set, w, r, false, failed);
                if (failed) br.status[k] = xg::BST_NOT_CONVERGED;
                std::copy(r.gradient.begin(), r.gradient.end(), br.gradient.begin() + 3 * (size_t)n * k);
                std::copy(r.dipole.begin(), r.dipole.end(), br.dipole.begin() + 3 * k);
            }
        } else {
            xg::run_batch(mols, set, std::vector<int>(mols.size(), 1), br, &guesses);
        }
        const int N3 = 3 * n;
        std::vector<double> H((size_t)N3 * N3, 0.0);
        int bad = 0;
        for (int ii = 0; ii < N3; ++ii) {
            const int r = 2 * ii, l = 2 * ii + 1;
            bad += (br.status[r] != xg::BST_OK) + (br.status[l] != xg::BST_OK);
            const double* gr = br.gradient.data() + 3 * (size_t)n * r;   // all molecules have n atoms
            const double* gl = br.gradient.data() + 3 * (size_t)n * l;
            for (int jj = 0; jj < N3; ++jj) H[(size_t)ii * N3 + jj] = (gr[jj] - gl[jj]) * step2;
            if (dipole_gradient)
                for (int x = 0; x < 3; ++x)
                    dipole_gradient[3 * ii + x] = (br.dipole[3 * (size_t)r + x] - br.dipole[3 * (size_t)l + x]) * step2;
        }
        for (int i = 0; i < N3; ++i)
            for (int j = i + 1; j < N3; ++j) {
                const double v = 0.5 * (H[(size_t)i * N3 + j] + H[(size_t)j * N3 + i]);
                H[(size_t)i * N3 + j] = v;
                H[(size_t)j * N3 + i] = v;
            }
        std::copy(H.begin(), H.end(), hessian);
        if (bad) env->error("Self consistent charge iterator did not converge", "scf");
    } catch (const std::exception& e) {
        env->error(e.what(), src);
    }
}

void xtb_cpcmx_calc(xtb_TEnvironment env, xtb_TMolecule, xtb_TCalculator, xtb_TResults) {
    if (!check_env(env)) return;
    env->error("CPCM-X solvation is not supported by this engine", "xtb_api_cpcmx_calc");
}

// ------------------------------------------------------------------ results
xtb_TResults xtb_newResults(void) { return new _xtb_TResults(); }

void xtb_delResults(xtb_TResults* res) {
    if (res && *res) {
        delete *res;
        *res = nullptr;
    }
}

xtb_TResults xtb_copyResults(xtb_TResults res) {
    if (!res) return nullptr;
    return new _xtb_TResults(*res);
}

static bool res_ready(xtb_TEnvironment env, xtb_TResults res, const char* src, const char* what) {
    if (!check_env(env)) return false;
    if (!res) {
        env->error("Results object is not allocated", src);
        return false;
    }
    if (!res->has) {
        env->error(std::string(what) + " is not available in results", src);
        return false;
    }
    return true;
}

void xtb_getEnergy(xtb_TEnvironment env, xtb_TResults res, double* energy) {
    if (!res_ready(env, res, "xtb_api_getEnergy", "Energy") || !energy) return;
    *energy = res->sp.energy;
}

void xtb_getGradient(xtb_TEnvironment env, xtb_TResults res, double* grad) {
    if (!res_ready(env, res, "xtb_api_getGradient", "Gradient") || !grad) return;
    std::copy(res->sp.gradient.begin(), res->sp.gradient.end(), grad);
}

void xtb_getSolvationEnergy(xtb_TEnvironment env, xtb_TResults res, double* energy) {
    if (!check_env(env)) return;
    if (!res) {
        env->error("Results object is not allocated", "xtb_api_getSolvationEnergy");
        return;
    }
    (void)energy;
    env->error("Solvation energy is not available in results", "xtb_api_getSolvationEnergy");
}

void xtb_getPCGradient(xtb_TEnvironment env, xtb_TResults res, double* grad) {
    if (!check_env(env)) return;
    if (!res) {
        env->error("Results object is not allocated", "xtb_api_getPCGradient");
        return;
    }
    if (!res->has || res->sp.pcgrad.empty()) {
        env->error("External charge gradients are not available in results", "xtb_api_getPCGradient");
        return;
    }
    if (grad) std::copy(res->sp.pcgrad.begin(), res->sp.pcgrad.end(), grad);
}

void xtb_getVirial(xtb_TEnvironment env, xtb_TResults res, double* virial) {
    if (!res_ready(env, res, "xtb_api_getVirial", "Virial") || !virial) return;
    for (int k = 0; k < 9; ++k) virial[k] = 0.0;
    for (int a = 0; a < res->nat; ++a)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) virial[3 * i + j] += res->xyz[3 * a + i] * res->sp.gradient[3 * a + j];
}

void xtb_getCharges(xtb_TEnvironment env, xtb_TResults res, double* charges) {
    if (!res_ready(env, res, "xtb_api_getCharges", "Partial charges") || !charges) return;
    std::copy(res->wfn.q.begin(), res->wfn.q.end(), charges);
}

void xtb_getDipole(xtb_TEnvironment env, xtb_TResults res, double* dipole) {
    if (!res_ready(env, res, "xtb_api_getDipole", "Dipole moment") || !dipole) return;
    std::copy(res->sp.dipole.begin(), res->sp.dipole.end(), dipole);
}

// Wiberg-Mayer bond orders (get_wiberg, src/scc_core.f90:1208-1245), evaluated on the device
void xtb_getBondOrders(xtb_TEnvironment env, xtb_TResults res, double* wbo) {
    if (!res_ready(env, res, "xtb_api_getBondOrders", "Bond orders") || !wbo) return;
    if (res->sp.wbo.empty()) {
        env->error("Bond orders are not available in results", "xtb_api_getBondOrders");
        return;
    }
    std::copy(res->sp.wbo.begin(), res->sp.wbo.end(), wbo);
}

void xtb_getNao(xtb_TEnvironment env, xtb_TResults res, int* nao) {
    if (!res_ready(env, res, "xtb_api_getNao", "Orbitals") || !nao) return;
    *nao = res->wfn.nao;
}

void xtb_getOrbitalEigenvalues(xtb_TEnvironment env, xtb_TResults res, double* emo) {
    if (!res_ready(env, res, "xtb_api_getOrbitalEigenvalues", "Orbital eigenvalues") || !emo) return;
    std::copy(res->wfn.emo.begin(), res->wfn.emo.end(), emo);
}

void xtb_getOrbitalOccupations(xtb_TEnvironment env, xtb_TResults res, double* focc) {
    if (!res_ready(env, res, "xtb_api_getOrbitalOccupations", "Orbital occupations") || !focc) return;
    std::copy(res->wfn.focc.begin(), res->wfn.focc.end(), focc);
}

void xtb_getOrbitalCoefficients(xtb_TEnvironment env, xtb_TResults res, double* c) {
    if (!res_ready(env, res, "xtb_api_getOrbitalCoefficients", "Orbital coefficients") || !c) return;
    if (res->wfn.C.empty()) {
        env->error("Orbital coefficients are not available in results", "xtb_api_getOrbitalCoefficients");
        return;
    }
    // the reference returns the Fortran array C(nao, nao) (AO index fastest), i.e. MO-major in C order
    const int n = res->wfn.nao;
    for (int mo = 0; mo < n; ++mo)
        for (int mu = 0; mu < n; ++mu) c[(size_t)mo * n + mu] = res->wfn.C[(size_t)mu * n + mo];
}

}  // extern "C"

// ------------------------------------------------------------------ engine extensions (xtb_gb300.h)
extern "C" {

int xtbgb_deviceCount(void) { return xg::device_count(); }

void xtbgb_fp64LatencyCycles(double* cycles) {
    if (!cycles) return;
    for (int k = 0; k < 5; ++k) cycles[k] = 0.0;
    if (xg::device_count() == 0) return;
    try {
        xg::fp64_latency_cycles(cycles);
    } catch (const std::exception&) {
    }
}

int xtbgb_reciprocalCheck(double* out) {
    if (!out) return 1;
    out[0] = out[1] = 0.0;
    if (xg::device_count() == 0) return 2;
    try {
        xg::reciprocal_check(out);
    } catch (const std::exception&) {
        return 3;
    }
    return 0;
}

int xtbgb_splitGemmCheck(int M, int N, int K, int slices, int seed, int exp_range, double* out) {
    if (!out || M < 1 || N < 1 || K < 1 || slices < 4 || slices > 7) return 1;
    if (xg::device_count() == 0) return 2;
    try {
        xg::split_gemm_check(M, N, K, slices, (unsigned)seed, exp_range, out);
    } catch (const std::exception&) {
        return 3;
    }
    return 0;
}

double xtbgb_fp64PeakTflops(void) {
    if (xg::device_count() == 0) return 0.0;
    try {
        return xg::fp64_peak_tflops();
    } catch (const std::exception&) {
        return 0.0;
    }
}

void xtbgb_fp64PeakDetail(double* out) {
    if (!out) return;
    for (int k = 0; k < 3; ++k) out[k] = 0.0;
    if (xg::device_count() == 0) return;
    try {
        xg::fp64_peak_tflops();
        xg::fp64_peak_detail(out);
    } catch (const std::exception&) {
    }
}

namespace {
// records of a Fortran unformatted sequential file: a 4-byte length before and after each
// record (the layout gfortran writes)
bool put_record(FILE* f, const void* p, size_t bytes) {
    const int32_t len = (int32_t)bytes;
    return fwrite(&len, 4, 1, f) == 1 && (bytes == 0 || fwrite(p, 1, bytes, f) == bytes) && fwrite(&len, 4, 1, f) == 1;
}

bool get_record(FILE* f, std::vector<char>& buf) {
    int32_t a = 0, b = 0;
    if (fread(&a, 4, 1, f) != 1 || a < 0) return false;
    buf.resize((size_t)a);
    if (a > 0 && fread(buf.data(), 1, (size_t)a, f) != (size_t)a) return false;
    return fread(&b, 4, 1, f) == 1 && a == b;
}
}  // namespace

// Restart file of the reference (writeRestart / readRestart, src/restart.f90:33-86, 182-200):
// a record of six 64-bit integers (method twice, atoms, shells, electrons, unpaired electrons),
// the shell charges, then for GFN2 the atomic dipoles (3, atoms) and quadrupoles (6, atoms).
int xtbgb_writeRestart(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TResults res, const char* filename) {
    static const char* src = "xtbgb_writeRestart";
    if (!check_env(env)) return 0;
    if (!mol || !res || !filename) {
        env->error("Molecule, results or file name missing", src);
        return 0;
    }
    xg::HostMol hm;
    const std::string err = xg::build_host_mol(mol->nat, mol->Z.data(), mol->xyz.data(), mol->charge, mol->uhf, hm);
    if (!err.empty()) {
        env->error(err, src);
        return 0;
    }
    const xg::Wavefunction& w = res->wfn;
    if (!w.valid() || w.nat != hm.nat || w.nsh != hm.nsh) {
        env->error("Results hold no wavefunction of this molecule", src);
        return 0;
    }
    FILE* f = fopen(filename, "wb");
    if (!f) {
        env->error(std::string("Could not open '") + filename + "' for writing", src);
        return 0;
    }
    const int64_t head[6] = {2, 2, hm.nat, hm.nsh, hm.nel, hm.nel_a - hm.nel_b};
    const bool ok = put_record(f, head, sizeof(head)) && put_record(f, w.qsh.data(), w.qsh.size() * 8) &&
                    put_record(f, w.dipm.data(), w.dipm.size() * 8) && put_record(f, w.qp.data(), w.qp.size() * 8);
    fclose(f);
    if (!ok) {
        env->error(std::string("Could not write '") + filename + "'", src);
        return 0;
    }
    return 1;
}

int xtbgb_readRestart(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TResults res, const char* filename) {
    static const char* src = "restart_readRestart";
    if (!check_env(env)) return 0;
    if (!mol || !res || !filename) {
        env->error("Molecule, results or file name missing", src);
        return 0;
    }
    xg::HostMol hm;
    const std::string err = xg::build_host_mol(mol->nat, mol->Z.data(), mol->xyz.data(), mol->charge, mol->uhf, hm);
    if (!err.empty()) {
        env->error(err, src);
        return 0;
    }
    FILE* f = fopen(filename, "rb");
    if (!f) return 0;   // no restart file: the reference goes on silently
    std::vector<char> rec;
    int64_t head[6] = {0, 0, 0, 0, 0, 0};
    if (!get_record(f, rec) || rec.size() != sizeof(head)) {
        fclose(f);
        env->warning("Dimension missmatch in restart file.", src);
        return 0;
    }
    std::memcpy(head, rec.data(), sizeof(head));
    if (head[0] != 2) env->warning("Version number missmatch in restart file.", src);
    if (head[4] != hm.nel) env->warning("Number of electron missmatch in restart file.", src);
    if (head[5] != hm.nel_a - hm.nel_b) env->warning("Multiplicity missmatch in restart file.", src);
    if (head[2] != hm.nat || head[3] != hm.nsh) {
        fclose(f);
        env->warning("Dimension missmatch in restart file.", src);
        return 0;
    }
    xg::Wavefunction w;
    w.nat = hm.nat;
    w.nao = hm.nao;
    w.nsh = hm.nsh;
    w.qsh.assign(hm.nsh, 0.0);
    w.dipm.assign(3 * (size_t)hm.nat, 0.0);
    w.qp.assign(6 * (size_t)hm.nat, 0.0);
    bool ok = get_record(f, rec) && rec.size() == w.qsh.size() * 8;
    if (ok) std::memcpy(w.qsh.data(), rec.data(), rec.size());
    if (ok && head[0] > 1) {   // GFN2 files carry the cumulative atomic multipoles
        ok = get_record(f, rec) && rec.size() == w.dipm.size() * 8;
        if (ok) std::memcpy(w.dipm.data(), rec.data(), rec.size());
        ok = ok && get_record(f, rec) && rec.size() == w.qp.size() * 8;
        if (ok) std::memcpy(w.qp.data(), rec.data(), rec.size());
    }
    fclose(f);
    if (!ok) {
        env->warning("Dimension missmatch in restart file.", src);
        return 0;
    }
    w.q.assign(hm.nat, 0.0);
    for (int s = 0; s < hm.nsh; ++s) w.q[hm.sh_atom[s]] += w.qsh[s];
    res->wfn = std::move(w);
    return 1;
}

void xtbgb_setExternalChargesHardness(xtb_TEnvironment env, xtb_TCalculator calc, int n, const double* charges,
                                      const double* positions, const double* hardness) {
    if (!check_env(env)) return;
    if (!hardness) {
        env->error("Hardness values are missing", "xtbgb_setExternalChargesHardness");
        return;
    }
    set_external_charges(env, calc, n, nullptr, charges, positions, hardness, "xtbgb_setExternalChargesHardness");
}

double xtbgb_sytrdMs(xtb_TEnvironment env, int n, int form, int max_blocks, int reps) {
    static const char* src = "xtbgb_sytrdMs";
    if (!check_env(env)) return -1.0;
    if (xg::device_count() == 0) {
        env->error("no CUDA device available for the GFN2 engine", src);
        return -1.0;
    }
    if (n < 3 || n > 8192 || form < -1 || form > 1) {
        env->error("n must lie in 3..8192 and form in -1..1", src);
        return -1.0;
    }
    try {
        return xg::time_sytrd(n, form, max_blocks, reps);
    } catch (const std::exception& e) {
        env->error(e.what(), src);
        return -1.0;
    }
}

int xtbgb_backtransformCheck(xtb_TEnvironment env, int n, int ncol, int slices, double* out) {
    static const char* src = "xtbgb_backtransformCheck";
    if (!check_env(env)) return 1;
    if (xg::device_count() == 0) {
        env->error("no CUDA device available for the GFN2 engine", src);
        return 1;
    }
    if (!out || n < 3 || n > 8192 || ncol < 1 || ncol > n || slices < 0 || slices > 8) {
        env->error("n must lie in 3..8192, ncol in 1..n and slices in 0..8 (out not null)", src);
        return 1;
    }
    try {
        xg::check_backtransform(n, ncol, slices, out);
        return 0;
    } catch (const std::exception& e) {
        env->error(e.what(), src);
        return 1;
    }
}

int xtbgb_autotune(xtb_TEnvironment env, double* out, int nout) {
    static const char* src = "xtbgb_autotune";
    if (!check_env(env)) return 0;
    if (xg::device_count() == 0) {
        env->error("no CUDA device available for the GFN2 engine", src);
        return 0;
    }
    try {
        const xg::Tuned t = xg::autotune();
        std::vector<double> v = {(double)t.sytrd_sym_min, (double)t.blocked_min_fp64, (double)t.blocked_min_split,
                                 t.seconds, (double)(t.sytrd_rows.size() / 3)};
        v.insert(v.end(), t.sytrd_rows.begin(), t.sytrd_rows.end());
        v.push_back((double)(t.backtr_rows.size() / 4));
        v.insert(v.end(), t.backtr_rows.begin(), t.backtr_rows.end());
        const int m = std::min((int)v.size(), std::max(0, nout));
        if (out) std::copy(v.begin(), v.begin() + m, out);
        return m;
    } catch (const std::exception& e) {
        env->error(e.what(), src);
        return 0;
    }
}

void xtbgb_getTuning(xtb_TEnvironment env, double* out) {
    if (!check_env(env) || !out) return;
    const xg::Tuned t = xg::tuned();
    out[0] = t.sytrd_sym_min;
    out[1] = t.blocked_min_fp64;
    out[2] = t.blocked_min_split;
    out[3] = t.level;
}

void xtbgb_setTuning(xtb_TEnvironment env, int sytrd_sym_min, int blocked_min_fp64, int blocked_min_split) {
    if (!check_env(env)) return;
    xg::set_tuned(std::max(3, sytrd_sym_min), std::max(0, blocked_min_fp64), std::max(0, blocked_min_split));
}

void xtbgb_getIterations(xtb_TEnvironment env, xtb_TResults res, int* iterations, int* converged) {
    if (!res_ready(env, res, "xtbgb_getIterations", "SCC information")) return;
    if (iterations) *iterations = res->sp.iterations;
    if (converged) *converged = res->sp.converged ? 1 : 0;
}

void xtbgb_getEnergyParts(xtb_TEnvironment env, xtb_TResults res, double* parts) {
    if (!res_ready(env, res, "xtbgb_getEnergyParts", "Energy parts") || !parts) return;
    const auto& s = res->sp;
    const double v[8] = {s.e_elec, s.e_rep, s.e_es, s.e_aes, s.e_axc, s.e_disp, s.e_atm, s.hl_gap};
    std::copy(v, v + 8, parts);
}

int xtbgb_getSolvationEnergyParts(xtb_TEnvironment env, xtb_TResults res, double* parts) {
    if (!res_ready(env, res, "xtbgb_getSolvationEnergyParts", "Solvation energy") || !parts) return 0;
    const auto& s = res->sp;
    const double v[5] = {s.g_solv, s.g_born, s.g_hb, s.g_sasa, s.g_shift};
    std::copy(v, v + 5, parts);
    return s.solvated ? 1 : 0;
}

void xtbgb_setSolventKernel(xtb_TEnvironment env, xtb_TCalculator calc, int kernel) {
    static const char* src = "xtbgb_setSolventKernel";
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", src);
        return;
    }
    const xg::SolventSpec& cur = calc->set.solv;
    if (!cur.on) {
        env->error("No solvation model set", src);
        return;
    }
    if (kernel != 0 && kernel != 1) {
        env->error("Unknown Born kernel (0 Still, 1 P16)", src);
        return;
    }
    if (kernel == 1 && cur.ion_strength > 0.0) {
        env->error("Salt screening needs the GBSA (Still) kernel", src);
        return;
    }
    xg::SolventSpec spec;
    const std::string err = xg::make_solvent_spec(cur.solvent, cur.alpb ? "alpb" : "gbsa", cur.state, cur.temperature,
                                                  cur.nang, spec, kernel);
    if (!err.empty()) {
        env->error(err, src);
        return;
    }
    spec.ion_strength = cur.ion_strength;
    spec.ion_rad = cur.ion_rad;
    calc->set.solv = spec;
}

void xtbgb_setSolventSalt(xtb_TEnvironment env, xtb_TCalculator calc, double ion_strength, double ion_rad) {
    static const char* src = "xtbgb_setSolventSalt";
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", src);
        return;
    }
    if (!(ion_strength >= 0.0) || !(ion_rad >= 0.0) || !std::isfinite(ion_strength) || !std::isfinite(ion_rad)) {
        env->error("Ion strength and ion radius must be finite and not negative", src);
        return;
    }
    if (calc->set.solv.on && calc->set.solv.kernel != 0 && ion_strength > 0.0) {
        env->error("Salt screening needs the GBSA (Still) kernel", src);
        return;
    }
    calc->set.solv.ion_strength = ion_strength;
    calc->set.solv.ion_rad = ion_rad;
}

void xtbgb_getPhaseTimes(xtb_TEnvironment env, xtb_TResults res, double* ms) {
    if (!res_ready(env, res, "xtbgb_getPhaseTimes", "Timings") || !ms) return;
    for (int k = 0; k < xg::PH_COUNT; ++k) ms[k] = k < (int)res->sp.phase_ms.size() ? res->sp.phase_ms[k] : 0.0;
}

void xtbgb_getTransferBytes(xtb_TEnvironment env, xtb_TResults res, long long* bytes) {
    if (!res_ready(env, res, "xtbgb_getTransferBytes", "Transfer statistics") || !bytes) return;
    bytes[0] = res->sp.h2d_bytes;
    bytes[1] = res->sp.d2h_bytes;
    bytes[2] = res->sp.launches;
}

void xtbgb_setPrecision(xtb_TEnvironment env, xtb_TCalculator calc, int split, int slices) {
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", "xtbgb_setPrecision");
        return;
    }
    if (split && (slices < 4 || slices > 7)) {
        env->error("Split precision needs 4..7 slices", "xtbgb_setPrecision");
        return;
    }
    calc->set.precision = split ? 1 : 0;
    calc->set.slices = slices;
}

void xtbgb_setBlockedBacktransform(xtb_TEnvironment env, xtb_TCalculator calc, int nao_min) {
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", "xtbgb_setBlockedBacktransform");
        return;
    }
    if (nao_min < -1) {
        env->error("AO threshold must be -1 (by precision) or >= 0", "xtbgb_setBlockedBacktransform");
        return;
    }
    calc->set.blocked_min = nao_min;
}

void xtbgb_setKeepOrbitals(xtb_TEnvironment env, xtb_TCalculator calc, int keep) {
    if (!check_env(env)) return;
    if (!calc) {
        env->error("Singlepoint calculator is not allocated", "xtbgb_setKeepOrbitals");
        return;
    }
    calc->keep_orbitals = keep != 0;
}

void xtbgb_getShellCharges(xtb_TEnvironment env, xtb_TResults res, double* qsh) {
    if (!res_ready(env, res, "xtbgb_getShellCharges", "Shell charges") || !qsh) return;
    std::copy(res->wfn.qsh.begin(), res->wfn.qsh.end(), qsh);
}

void xtbgb_getMultipoles(xtb_TEnvironment env, xtb_TResults res, double* dipm, double* qp) {
    if (!res_ready(env, res, "xtbgb_getMultipoles", "Multipoles")) return;
    if (dipm) std::copy(res->wfn.dipm.begin(), res->wfn.dipm.end(), dipm);
    if (qp) std::copy(res->wfn.qp.begin(), res->wfn.qp.end(), qp);
}


// ------------------------------------------------------------------ batched single points
struct _xtbgb_TBatch {
    int nmol = 0;
    std::vector<int> natoms;
    std::vector<long> atom_off;
    std::vector<xg::HostMol> mols;
    xg::BatchResults res;
    bool has = false;
};

xtbgb_TBatch xtbgb_newBatch(xtb_TEnvironment env, int nmol, const int* natoms, const int* numbers,
                            const double* positions, const double* charges, const int* uhf) {
    static const char* src = "xtbgb_newBatch";
    if (!check_env(env)) return nullptr;
    if (nmol < 0 || (nmol > 0 && (!natoms || !numbers || !positions))) {
        env->error("Invalid batch description", src);
        return nullptr;
    }
    auto* b = new _xtbgb_TBatch();
    b->nmol = nmol;
    b->natoms.assign(natoms, natoms + nmol);
    b->atom_off.assign(nmol + 1, 0);
    for (int i = 0; i < nmol; ++i) {
        if (natoms[i] < 1) {
            env->error("Molecule " + std::to_string(i) + " has no atoms", src);
            delete b;
            return nullptr;
        }
        b->atom_off[i + 1] = b->atom_off[i] + natoms[i];
    }
    b->mols.resize(nmol);
    for (int i = 0; i < nmol; ++i) {
        const long o = b->atom_off[i];
        for (int a = 0; a < natoms[i]; ++a)
            if (numbers[o + a] < 1 || numbers[o + a] > kMaxElem) {
                env->error("Molecule " + std::to_string(i) + ": element " + std::to_string(numbers[o + a]) +
                               " is not parametrised in GFN2-xTB", src);
                delete b;
                return nullptr;
            }
        const std::string err = xg::build_host_mol(natoms[i], numbers + o, positions + 3 * o,
                                                   charges ? charges[i] : 0.0, uhf ? uhf[i] : 0, b->mols[i]);
        if (!err.empty()) {
            env->error("Molecule " + std::to_string(i) + ": " + err, src);
            delete b;
            return nullptr;
        }
    }
    return b;
}

void xtbgb_delBatch(xtbgb_TBatch* batch) {
    if (batch && *batch) {
        delete *batch;
        *batch = nullptr;
    }
}

void xtbgb_batchSinglepoint(xtb_TEnvironment env, xtbgb_TBatch batch, double accuracy, double etemp, int maxiter,
                            int gradient) {
    static const char* src = "xtbgb_batchSinglepoint";
    if (!check_env(env)) return;
    if (!batch) {
        env->error("Batch is not allocated", src);
        return;
    }
    xg::BatchSettings set;
    set.accuracy = std::min(std::max(accuracy, 1.0e-4), 1.0e3);
    set.etemp = std::max(etemp, 1.0e-6);
    set.maxiter = std::max(maxiter, 1);
    std::vector<int> wg(batch->nmol, gradient ? 1 : 0);
    try {
        xg::run_batch(batch->mols, set, wg, batch->res);
    } catch (const std::exception& e) {
        env->error(e.what(), src);
        batch->has = false;
        return;
    }
    batch->has = true;
    int bad = 0;
    for (int i = 0; i < batch->nmol; ++i) bad += batch->res.status[i] != xg::BST_OK;
    if (bad) env->error(std::to_string(bad) + " molecule(s) failed or did not converge (see xtbgb_batchGetStatus)", src);
}

static bool batch_ready(xtb_TEnvironment env, xtbgb_TBatch batch, const char* src) {
    if (!check_env(env)) return false;
    if (!batch || !batch->has) {
        env->error("Batch results are not available", src);
        return false;
    }
    return true;
}

void xtbgb_batchGetEnergies(xtb_TEnvironment env, xtbgb_TBatch batch, double* energies) {
    if (!batch_ready(env, batch, "xtbgb_batchGetEnergies") || !energies) return;
    std::copy(batch->res.energy.begin(), batch->res.energy.end(), energies);
}

void xtbgb_batchGetGradients(xtb_TEnvironment env, xtbgb_TBatch batch, double* gradients) {
    if (!batch_ready(env, batch, "xtbgb_batchGetGradients") || !gradients) return;
    std::copy(batch->res.gradient.begin(), batch->res.gradient.end(), gradients);
}

void xtbgb_batchGetCharges(xtb_TEnvironment env, xtbgb_TBatch batch, double* charges) {
    if (!batch_ready(env, batch, "xtbgb_batchGetCharges") || !charges) return;
    std::copy(batch->res.charges.begin(), batch->res.charges.end(), charges);
}

void xtbgb_batchGetDipoles(xtb_TEnvironment env, xtbgb_TBatch batch, double* dipoles) {
    if (!batch_ready(env, batch, "xtbgb_batchGetDipoles") || !dipoles) return;
    std::copy(batch->res.dipole.begin(), batch->res.dipole.end(), dipoles);
}

void xtbgb_batchGetEnergyParts(xtb_TEnvironment env, xtbgb_TBatch batch, double* parts) {
    if (!batch_ready(env, batch, "xtbgb_batchGetEnergyParts") || !parts) return;
    std::copy(batch->res.parts.begin(), batch->res.parts.end(), parts);
}

void xtbgb_batchGetStatus(xtb_TEnvironment env, xtbgb_TBatch batch, int* iterations, int* converged, int* status,
                          int* engine) {
    if (!batch_ready(env, batch, "xtbgb_batchGetStatus")) return;
    const auto& r = batch->res;
    if (iterations) std::copy(r.iterations.begin(), r.iterations.end(), iterations);
    if (converged) std::copy(r.converged.begin(), r.converged.end(), converged);
    if (status) std::copy(r.status.begin(), r.status.end(), status);
    if (engine) std::copy(r.engine.begin(), r.engine.end(), engine);
}

void xtbgb_batchGetStats(xtb_TEnvironment env, xtbgb_TBatch batch, double* times, long long* counts) {
    if (!batch_ready(env, batch, "xtbgb_batchGetStats")) return;
    const auto& r = batch->res;
    if (times) {
        times[0] = r.device_ms;
        times[1] = r.wall_ms;
    }
    if (counts) {
        counts[0] = r.h2d;
        counts[1] = r.d2h;
        counts[2] = r.launches;
        counts[3] = r.plain_count;
    }
}

void xtbgb_batchNao(xtb_TEnvironment env, xtbgb_TBatch batch, int* nao) {
    if (!check_env(env) || !batch || !nao) return;
    for (int i = 0; i < batch->nmol; ++i) nao[i] = batch->mols[i].nao;
}


// ------------------------------------------------------------------ request loop
struct _xtbgb_TServer {
    std::unique_ptr<xg::Server> srv;
};

xtbgb_TServer xtbgb_newServer(xtb_TEnvironment env, double pool_gib, int max_slots, int plain_workers,
                              int iters_per_step, double accuracy, double etemp, int maxiter) {
    return xtbgb_newServerEx(env, pool_gib, max_slots, plain_workers, iters_per_step, accuracy, etemp, maxiter, 0, 5,
                             0, 0);
}

xtbgb_TServer xtbgb_newServerEx(xtb_TEnvironment env, double pool_gib, int max_slots, int plain_workers,
                                int iters_per_step, double accuracy, double etemp, int maxiter, int split,
                                int slices, int pool_max_nao, int coop_blocks) {
    static const char* src = "xtbgb_newServer";
    if (!check_env(env)) return nullptr;
    xg::ServeConfig cfg;
    cfg.pool_bytes = (size_t)(std::max(pool_gib, 0.01) * (double)(size_t(1) << 30));
    cfg.max_slots = std::max(1, max_slots);
    cfg.plain_workers = std::max(1, plain_workers);
    cfg.iters_per_step = std::max(1, iters_per_step);
    cfg.set.accuracy = std::min(std::max(accuracy, 1.0e-4), 1.0e3);
    cfg.set.etemp = std::max(etemp, 1.0e-6);
    cfg.set.maxiter = std::max(maxiter, 1);
    if (split && (slices < 4 || slices > 7)) {
        env->error("Split precision needs 4..7 slices", src);
        return nullptr;
    }
    cfg.precision = split ? 1 : 0;
    cfg.slices = slices;
    cfg.pool_max_nao = pool_max_nao > 0 ? std::min(pool_max_nao, xg::BATCH_MAX_NAO) : xg::BATCH_MAX_NAO;
    cfg.coop_blocks = coop_blocks;
    auto* s = new _xtbgb_TServer();
    try {
        s->srv = std::make_unique<xg::Server>(cfg);
    } catch (const std::exception& e) {
        env->error(e.what(), src);
        delete s;
        return nullptr;
    }
    return s;
}

void xtbgb_delServer(xtbgb_TServer* srv) {
    if (srv && *srv) {
        delete *srv;
        *srv = nullptr;
    }
}

long long xtbgb_serverSubmit(xtb_TEnvironment env, xtbgb_TServer srv, int natoms, const int* numbers,
                             const double* positions, double charge, int uhf, int gradient) {
    static const char* src = "xtbgb_serverSubmit";
    if (!check_env(env)) return -1;
    if (!srv || !srv->srv) {
        env->error("Server is not allocated", src);
        return -1;
    }
    if (natoms < 1 || !numbers || !positions) {
        env->error("Invalid molecule", src);
        return -1;
    }
    for (int a = 0; a < natoms; ++a)
        if (numbers[a] < 1 || numbers[a] > kMaxElem) {
            env->error("Element " + std::to_string(numbers[a]) + " is not parametrised in GFN2-xTB", src);
            return -1;
        }
    std::string err;
    const long long id = srv->srv->submit(natoms, numbers, positions, charge, uhf, gradient, err);
    if (id < 0) env->error(err, src);
    return id;
}

int xtbgb_serverWait(xtb_TEnvironment env, xtbgb_TServer srv, long long id, double timeout, double* energy,
                     double* gradient, double* charges, double* info) {
    static const char* src = "xtbgb_serverWait";
    if (!check_env(env)) return 0;
    if (!srv || !srv->srv) {
        env->error("Server is not allocated", src);
        return 0;
    }
    xg::Completed c;
    if (!srv->srv->wait(id, c, timeout)) return 0;
    if (energy) *energy = c.energy;
    if (gradient) std::copy(c.gradient.begin(), c.gradient.end(), gradient);
    if (charges) std::copy(c.charges.begin(), c.charges.end(), charges);
    if (info) {
        info[0] = c.iterations;
        info[1] = c.converged;
        info[2] = c.status;
        info[3] = c.engine;
        info[4] = c.t_submit;
        info[5] = c.t_start;
        info[6] = c.t_done;
        info[7] = c.dipole[0];
        info[8] = c.dipole[1];
        info[9] = c.dipole[2];
        info[10] = c.nao;
        info[11] = c.sytrd_ms;
    }
    if (!c.error.empty()) env->error(c.error, src);
    else if (c.status == xg::BST_CHOLESKY) env->error("Overlap matrix is not positive definite", src);
    else if (c.status == xg::BST_NONFINITE) env->error("Energy or gradient is not finite", src);
    else if (c.status != xg::BST_OK) env->error("Self consistent charge iterator did not converge", src);
    return 1;
}

void xtbgb_serverInjectAdmissionFailures(xtb_TEnvironment env, xtbgb_TServer srv, int count) {
    static const char* src = "xtbgb_serverInjectAdmissionFailures";
    if (!check_env(env)) return;
    if (!srv || !srv->srv) {
        env->error("Server is not allocated", src);
        return;
    }
    srv->srv->inject_admission_failures(count);
}

void xtbgb_serverStats(xtb_TEnvironment env, xtbgb_TServer srv, double* stats) {
    if (!check_env(env) || !srv || !srv->srv || !stats) return;
    const auto v = srv->srv->stats();
    std::copy(v.begin(), v.end(), stats);
}

}  // extern "C"
