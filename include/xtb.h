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
 * Only the GFN2-xTB Hamiltonian is implemented.  Entry points for other
 * methods and for solvation / external charges are exported and push an
 * "unsupported" error, as the reference does for unavailable features.
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
extern XTB_API_ENTRY void XTB_API_CALL
xtb_setSolvent(xtb_TEnvironment env, xtb_TCalculator calc, char* solvent, int* state, double* temp,
               int* grid, char* model);
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

/* ---- single point [ref include/xtb.h:236-240] ---- */
extern XTB_API_ENTRY void XTB_API_CALL
xtb_singlepoint(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TCalculator calc, xtb_TResults res);

/* ---- results [ref include/xtb.h:259-344] ---- */
extern XTB_API_ENTRY xtb_TResults XTB_API_CALL xtb_newResults(void);
extern XTB_API_ENTRY void XTB_API_CALL xtb_delResults(xtb_TResults* res);
extern XTB_API_ENTRY xtb_TResults XTB_API_CALL xtb_copyResults(xtb_TResults res);
extern XTB_API_ENTRY void XTB_API_CALL xtb_getEnergy(xtb_TEnvironment env, xtb_TResults res, double* energy);
/* gradient[natoms][3] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getGradient(xtb_TEnvironment env, xtb_TResults res, double* grad);
/* Mulliken partial charges[natoms] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getCharges(xtb_TEnvironment env, xtb_TResults res, double* charges);
/* dipole[3] in e*Bohr [ref include/xtb.h:277-280] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getDipole(xtb_TEnvironment env, xtb_TResults res, double* dipole);
/* Wiberg bond orders[natoms][natoms] [ref include/xtb.h:313-316] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getBondOrders(xtb_TEnvironment env, xtb_TResults res, double* wbo);
extern XTB_API_ENTRY void XTB_API_CALL xtb_getNao(xtb_TEnvironment env, xtb_TResults res, int* nao);
/* orbital energies[nao] in Hartree [ref include/xtb.h:325-328] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getOrbitalEigenvalues(xtb_TEnvironment env, xtb_TResults res, double* emo);
extern XTB_API_ENTRY void XTB_API_CALL xtb_getOrbitalOccupations(xtb_TEnvironment env, xtb_TResults res, double* focc);
/* coefficients[nao][nao] [ref include/xtb.h:337-340] */
extern XTB_API_ENTRY void XTB_API_CALL xtb_getOrbitalCoefficients(xtb_TEnvironment env, xtb_TResults res, double* c);

#ifdef __cplusplus
}
#endif
