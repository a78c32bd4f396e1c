/* Drop-in check: a plain C program driving libxtb_gb300.so exactly like the
 * reference's C API example drives libxtb (propyne, GFN2-xTB, 300 K, 30 iterations; then in
 * implicit water with GBSA and ALPB) and asserting the reference's published values. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "xtb.h"

static int check(double actual, double expected, double thr, const char* msg) {
    if (fabs(actual - expected) > thr) {
        printf("FAIL %s: %.14f vs %.14f (thr %.1e)\n", msg, actual, expected, thr);
        return 0;
    }
    return 1;
}

int main(void) {
    const int natoms = 7;
    const int attyp[7] = {6, 6, 6, 1, 1, 1, 1};
    const double coord[21] = {
        0.00000000000000,  0.00000000000000, -1.79755622305860,
        0.00000000000000,  0.00000000000000,  0.95338756106749,
        0.00000000000000,  0.00000000000000,  3.22281255790261,
       -0.96412815539807, -1.66991895015711, -2.53624948351102,
       -0.96412815539807,  1.66991895015711, -2.53624948351102,
        1.92825631079613,  0.00000000000000, -2.53624948351102,
        0.00000000000000,  0.00000000000000,  5.23010455462158};
    double energy, q[7], dipole[3], wbo[49], grad[21];
    char buffer[512];
    int bufsize = 512, ok = 1;

    if (xtb_getAPIVersion() != XTB_API_VERSION) return 1;
    xtb_TEnvironment env = xtb_newEnvironment();
    xtb_TCalculator calc = xtb_newCalculator();
    xtb_TResults res = xtb_newResults();
    xtb_TMolecule mol = xtb_newMolecule(env, &natoms, attyp, coord, NULL, NULL, NULL, NULL);
    if (xtb_checkEnvironment(env)) return 2;
    xtb_getEnergy(env, res, &energy);            /* no results yet: must be an error */
    if (!xtb_checkEnvironment(env)) return 3;
    xtb_getError(env, buffer, &bufsize);
    xtb_setVerbosity(env, XTB_VERBOSITY_MUTED);
    xtb_loadGFN2xTB(env, mol, calc, NULL);
    xtb_setAccuracy(env, calc, 1.0);
    xtb_setElectronicTemp(env, calc, 300.0);
    xtb_setMaxIter(env, calc, 30);
    if (xtb_checkEnvironment(env)) return 4;
    xtb_singlepoint(env, mol, calc, res);
    if (xtb_checkEnvironment(env)) {
        xtb_showEnvironment(env, "single point failed");
        return 5;
    }
    xtb_getEnergy(env, res, &energy);
    xtb_getCharges(env, res, q);
    xtb_getDipole(env, res, dipole);
    xtb_getBondOrders(env, res, wbo);
    xtb_getGradient(env, res, grad);
    if (xtb_checkEnvironment(env)) return 6;
    ok &= check(energy, -8.3824793849585, 1.0e-9, "energy");
    ok &= check(q[5], 0.05184019996829, 1.0e-8, "charge");
    ok &= check(dipole[2], -0.298279305689518, 1.0e-6, "dipole");
    ok &= check(wbo[9], 2.89823984265213, 1.0e-8, "bond order");
    ok &= check(grad[3 * 0 + 2], -0.74649908147372E-03, 1.0e-9, "gradient");
    /* implicit water, GBSA then ALPB, each started from the previous result (c_api_example.c:114-163) */
    {
        char solvent[] = "h2o", gbsa[] = "gbsa", alpb[] = "alpb", bogus[] = "unobtainium";
        xtb_setSolvent(env, calc, solvent, NULL, NULL, NULL, gbsa);
        xtb_singlepoint(env, mol, calc, res);
        xtb_getEnergy(env, res, &energy);
        xtb_getCharges(env, res, q);
        xtb_getDipole(env, res, dipole);
        xtb_getBondOrders(env, res, wbo);
        if (xtb_checkEnvironment(env)) return 9;
        ok &= check(energy, -8.38393864716134, 1.0e-9, "GBSA energy");
        ok &= check(q[5], 0.06090868805034, 1.0e-8, "GBSA charge");
        ok &= check(dipole[2], -0.35455233974705, 1.0e-6, "GBSA dipole");
        ok &= check(wbo[9], 2.89453979224265, 1.0e-8, "GBSA bond order");
        xtb_releaseSolvent(env, calc);
        xtb_setSolvent(env, calc, solvent, NULL, NULL, NULL, alpb);
        xtb_singlepoint(env, mol, calc, res);
        xtb_getEnergy(env, res, &energy);
        xtb_getCharges(env, res, q);
        xtb_getDipole(env, res, dipole);
        xtb_getBondOrders(env, res, wbo);
        if (xtb_checkEnvironment(env)) return 10;
        ok &= check(energy, -8.384076843892, 1.0e-9, "ALPB energy");
        ok &= check(q[5], 0.0644849340, 1.0e-8, "ALPB charge");
        ok &= check(dipole[2], -0.3641866008, 1.0e-6, "ALPB dipole");
        ok &= check(wbo[9], 2.8932146955, 1.0e-8, "ALPB bond order");
        xtb_releaseSolvent(env, calc);
        xtb_setSolvent(env, calc, bogus, NULL, NULL, NULL, gbsa);   /* not parametrized: an error */
        if (!xtb_checkEnvironment(env)) return 11;
    }
    xtb_delResults(&res);
    xtb_delCalculator(&calc);
    xtb_delMolecule(&mol);
    xtb_delEnvironment(&env);
    if (res || calc || mol || env) return 7;
    printf(ok ? "C API drop-in: all reference values reproduced\n" : "C API drop-in: mismatch\n");
    return ok ? 0 : 8;
}
