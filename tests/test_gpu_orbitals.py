"""Orbital getters of the drop-in against the oracle (needs a GB300).

xtb_getOrbitalEigenvalues returns emo in Hartree, xtb_getOrbitalOccupations the total
occupations and xtb_getOrbitalCoefficients the coefficient matrix with orbital j in the j-th
run of nao values, as the reference's getters do (src/api/results.f90:372-504).  Eigenvectors
are fixed only up to sign (and rotations inside degenerate sets), so the coefficients are
compared through the density they build, P = C^T diag(f) C, against the oracle's density.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import gfn2
from xtb_gb300 import interface as X
from xtb_gb300 import workloads as W

pytestmark = pytest.mark.gpu
EVTOAU = 1.0 / 27.21138505

CASES = {
    "propyne": ([6, 6, 6, 1, 1, 1, 1],
                [[0.0, 0.0, -1.79755622305860], [0.0, 0.0, 0.95338756106749], [0.0, 0.0, 3.22281255790261],
                 [-0.96412815539807, -1.66991895015711, -2.53624948351102],
                 [-0.96412815539807, 1.66991895015711, -2.53624948351102],
                 [1.92825631079613, 0.0, -2.53624948351102], [0.0, 0.0, 5.23010455462158]], 0, 0),
    "methyl_radical": ([6, 1, 1, 1], [[0, 0, 0], [2.04, 0, 0], [-1.02, 1.767, 0], [-1.02, -1.767, 0.05]], 0, 1),
    "water_cluster_10": W.water_cluster(10, seed=4) + (0, 0),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_orbital_getters_match_oracle(name):
    Z, xyz, charge, uhf = CASES[name]
    xyz = np.asarray(xyz, dtype=float)
    calc = X.Calculator(Z, xyz, charge=charge, uhf=uhf, keep_orbitals=True)
    r = calc.singlepoint()
    o = gfn2.singlepoint(Z, xyz, charge=charge, uhf=uhf)
    n = r.nao
    assert n == o.nao
    coef = np.zeros((n, n))
    calc.lib.xtb_getOrbitalCoefficients(calc.env.h, calc.res, coef.ctypes.data_as(C.POINTER(C.c_double)))
    calc.env.check()
    # eigenvalues (Hartree) and occupations
    assert np.max(np.abs(r.emo - o.emo * EVTOAU)) <= 1e-9
    assert np.max(np.abs(r.focc - o.focc)) <= 1e-8
    assert abs(np.sum(r.focc) - np.sum(o.focc)) <= 1e-9
    # every orbital is S-normalised: c_j^T S c_j = 1
    S = o.S
    assert np.max(np.abs(np.einsum("ji,ik,jk->j", coef, S, coef) - 1.0)) <= 1e-9
    # the density the orbitals build
    P = (coef.T * r.focc) @ coef
    assert np.max(np.abs(P - o.P)) <= 1e-7
