/*
 * xtb.h -- C ABI of the GB300 GFN2-xTB single-point engine (libxtb_gb300.so).
 *
 * Drop-in for the reference C API (xtb's include/xtb.h, API version 2.0.0):
 * every function below keeps the reference's symbol name, argument list,
 * argument meaning and error behaviour.  Each declaration cites the reference
 * declaration it replaces as  [ref include/xtb.h:<line>].
 *
 * Conventions shared with the reference:
 *  - handles are opaque pointers created by xtb_new* and released by xtb_del*,
 *    which also sets the caller's handle to NULL;
 *  - positions are Bohr, energies Hartree, gradients Hartree/Bohr;
 *  - functions never abort on bad input: errors are pushed onto the
 *    environment and are polled with xtb_checkEnvironment / xtb_getError;
 *    a NULL environment makes a call a silent no-op;
 *  - output arrays are caller-owned, getters copy into them.
 *
 * Only the GFN2-xTB Hamiltonian is implemented, with external point charges
 * and the GBSA / ALPB implicit solvents.  Entry points for the other methods
 * and solvent models (GFN0/GFN1/GFN-FF, COSMO, CPCM-X) are exported and push
 * an "unsupported" error, as the reference does for unavailable features.
 */
#pragma once

#define XTB_API_ENTRY
#define XTB_API_CALL
#define XTB_API_SUFFIX__VERSION_2_0_0

#define XTB_API_VERSION 20000

#define XTB_VERBOSITY_FULL    2
#define XTB_VERBOSITY_MINIMAL 1
#define XTB_VERBOSITY_MUTED   0

#ifdef __cplusplus
extern "C" {
#else
#include <stdbool.h>
#endif

typedef struct _xtb_TEnvironment* xtb_TEnvironment;   /* [ref include/xtb.h:55-58] */
typedef struct _xtb_TMolecule* xtb_TMolecule;         /* [ref include/xtb.h:59-60] */
typedef struct _xtb_TCalculator* xtb_TCalculator;     /* [ref include/xtb.h:61-62] */
typedef struct _xtb_TResults* xtb_TResults;           /* [ref include/xtb.h:63-64] */

#ifndef __cplusplus
/* Convenience deleter, as in the reference [ref include/xtb.h:37-42] */
#define xtb_delete(ptr) _Generic((ptr),               \
        xtb_TEnvironment: xtb_delEnvironment,          \
        xtb_TMolecule: xtb_delMolecule,                \
        xtb_TCalculator: xtb_delCalculator,            \
        xtb_TResults: xtb_delResults)(&ptr)
#endif

/* API version 10000*major + 100*minor + patch = 20000 [ref include/xtb.h:71-72] */
extern XTB_API_ENTRY int XTB_API_CALL xtb_getAPIVersion(void);

/* ---- environment: error log and output unit [ref include/xtb.h:79-113] ---- */
extern XTB_API_ENTRY xtb_TEnvironment XTB_API_CALL xtb_newEnvironment(void);
extern XTB_API_ENTRY void XTB_API_CALL xtb_delEnvironment(xtb_TEnvironment* env);
/* 0 = no error, 1 = errors pending */
extern XTB_API_ENTRY int XTB_API_CALL xtb_checkEnvironment(xtb_TEnvironment env);
/* print (with optional leading message) and clear the error log */
extern XTB_API_ENTRY void XTB_API_CALL xtb_showEnvironment(xtb_TEnvironment env, const char* message);
/* copy the error log into buffer[*buffersize] (NUL terminated) and clear it */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getError(xtb_TEnvironment env, char* buffer, const int* buffersize);
extern XTB_API_ENTRY void XTB_API_CALL xtb_setOutput(xtb_TEnvironment env, const char* filename);
extern XTB_API_ENTRY void XTB_API_CALL xtb_releaseOutput(xtb_TEnvironment env);
extern XTB_API_ENTRY void XTB_API_CALL xtb_setVerbosity(xtb_TEnvironment env, int verbosity);

/* ---- molecular structure [ref include/xtb.h:120-139] ---- */
/* natoms, numbers[natoms], positions[natoms][3] (Bohr); charge, uhf, lattice,
 * periodic may be NULL.  Periodic systems are rejected (molecules only). */
extern XTB_API_ENTRY xtb_TMolecule XTB_API_CALL
xtb_newMolecule(xtb_TEnvironment env, const int* natoms, const int* numbers, const double* positions,
                const double* charge, const int* uhf, const double* lattice, const bool* periodic);
extern XTB_API_ENTRY void XTB_API_CALL xtb_delMolecule(xtb_TMolecule* mol);
extern XTB_API_ENTRY void XTB_API_CALL
xtb_updateMolecule(xtb_TEnvironment env, xtb_TMolecule mol, const double* positions, const double* lattice);

/* ---- calculator [ref include/xtb.h:146-231] ---- */
extern XTB_API_ENTRY xtb_TCalculator XTB_API_CALL xtb_newCalculator(void);
extern XTB_API_ENTRY void XTB_API_CALL xtb_delCalculator(xtb_TCalculator* calc);
/* GFN2-xTB parametrisation; filename may be NULL (built-in parameter set) [ref include/xtb.h:168-172] */
extern XTB_API_ENTRY void XTB_API_CALL
xtb_loadGFN2xTB(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, char* filename);
/* unsupported methods: push an error [ref include/xtb.h:154-186] */
extern XTB_API_ENTRY void XTB_API_CALL
xtb_loadGFN0xTB(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, char* filename);
extern XTB_API_ENTRY void XTB_API_CALL
xtb_loadGFN1xTB(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, char* filename);
extern XTB_API_ENTRY void XTB_API_CALL
xtb_loadGFNFF(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, char* filename);
/* implicit solvent on a loaded calculator: solvent name (the reference's aliases, "none"/"gas"/"vac"
 * for none), solution state (NULL: 1 gsolv; 2 reference, 3 1 bar), temperature in K (NULL: 298.15),
 * Lebedev grid points per atom (NULL: 230) and model (NULL or "gbsa": Still kernel with the GBSA
 * parameters; "alpb": ALPB with the P16 kernel); "cosmo", "tmcosmo" and "cpcmx" push an error.
 * Unknown solvents push "solvent: '<name>' is not parametrized" and "Could not add solvation model
 * for '<name>'" [ref include/xtb.h:181-189] */
extern XTB_API_ENTRY void XTB_API_CALL
xtb_setSolvent(xtb_TEnvironment env, xtb_TCalculator calc, char* solvent, int* state, double* temp,
               int* grid, char* model);
/* back to the gas phase [ref include/xtb.h:191-195] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_releaseSolvent(xtb_TEnvironment env, xtb_TCalculator calc);
extern XTB_API_ENTRY void XTB_API_CALL
xtb_setExternalCharges(xtb_TEnvironment env, xtb_TCalculator calc, int* n, int* numbers, double* charges,
                       double* positions);
extern XTB_API_ENTRY void XTB_API_CALL xtb_releaseExternalCharges(xtb_TEnvironment env, xtb_TCalculator calc);
/* accuracy clamped to [1e-4, 1e3] [ref include/xtb.h:210-214] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_setAccuracy(xtb_TEnvironment env, xtb_TCalculator calc, double accuracy);
/* max SCC iterations, at least 1 [ref include/xtb.h:217-221] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_setMaxIter(xtb_TEnvironment env, xtb_TCalculator calc, int iterations);
/* electronic temperature in K, at least 1e-6 [ref include/xtb.h:224-228] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_setElectronicTemp(xtb_TEnvironment env, xtb_TCalculator calc, double temperature);

/* ---- single point [ref include/xtb.h:235-240] ---- */
extern XTB_API_ENTRY void XTB_API_CALL
xtb_singlepoint(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, xtb_TResults res);

/* Numerical Hessian [3N][3N] (Hartree/Bohr^2) by central differences of analytic gradients,
 * step 0.005 Bohr, every displaced point starting from the results object's wavefunction (a
 * fresh object: the initial guess of the undisplaced molecule); the displaced single points
 * run together on the batched engine.  dipole_gradient [3N][3] may be NULL.  The reference
 * header declares atom_index_list and step_size in this order while its implementation reads
 * a step and a list; both must be NULL here (all atoms, default step), as in the reference's
 * own C test.  Polarizability gradients are not computed (non-NULL raises an error).
 * [ref include/xtb.h:242-252] */
extern XTB_API_ENTRY void XTB_API_CALL
xtb_hessian(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, xtb_TResults res, double* hessian,
            int* atom_index_list, int* step_size, double* dipole_gradient, double* polarizability_gradient);

/* CPCM-X solvation: not supported, pushes an error [ref include/xtb.h:228-233] */
extern XTB_API_ENTRY void XTB_API_CALL
xtb_cpcmx_calc(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, xtb_TResults res);

/* ---- results [ref include/xtb.h:258-344] ---- */
extern XTB_API_ENTRY xtb_TResults XTB_API_CALL xtb_newResults(void);                       /* [ref :260] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_delResults(xtb_TResults* res);                  /* [ref :264] */
extern XTB_API_ENTRY xtb_TResults XTB_API_CALL xtb_copyResults(xtb_TResults res);           /* [ref :268] */
/* total energy in Hartree [ref include/xtb.h:272] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getEnergy(xtb_TEnvironment env, xtb_TResults res, double* energy);
/* pushes "Solvation energy is not available in results", as the reference does for every model but
 * CPCM-X (the GBSA / ALPB parts are read with xtbgb_getSolvationEnergyParts) [ref include/xtb.h:278] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getSolvationEnergy(xtb_TEnvironment env, xtb_TResults res, double* energy);
/* gradient[natoms][3] in Hartree/Bohr [ref include/xtb.h:284] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getGradient(xtb_TEnvironment env, xtb_TResults res, double* grad);
/* gradient[npc][3] on the external charges of the last single point; without charges pushes
 * "not available" [ref include/xtb.h:290] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getPCGradient(xtb_TEnvironment env, xtb_TResults res, double* grad);
/* virial[3][3] in Hartree: dE/d(strain) = sum_A R_A g_A^T of the molecule [ref include/xtb.h:296] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getVirial(xtb_TEnvironment env, xtb_TResults res, double* virial);
/* dipole[3] in e*Bohr [ref include/xtb.h:302] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getDipole(xtb_TEnvironment env, xtb_TResults res, double* dipole);
/* Mulliken partial charges[natoms] [ref include/xtb.h:308] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getCharges(xtb_TEnvironment env, xtb_TResults res, double* charges);
/* Wiberg bond orders[natoms][natoms] [ref include/xtb.h:314] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getBondOrders(xtb_TEnvironment env, xtb_TResults res, double* wbo);
/* number of atomic orbitals [ref include/xtb.h:320] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getNao(xtb_TEnvironment env, xtb_TResults res, int* nao);
/* orbital energies[nao] in Hartree [ref include/xtb.h:326] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getOrbitalEigenvalues(xtb_TEnvironment env, xtb_TResults res, double* emo);
/* orbital occupations[nao] [ref include/xtb.h:332] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getOrbitalOccupations(xtb_TEnvironment env, xtb_TResults res, double* focc);
/* coefficients[nao][nao] [ref include/xtb.h:338] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getOrbitalCoefficients(xtb_TEnvironment env, xtb_TResults res, double* c);

#ifdef __cplusplus
}
#endif
