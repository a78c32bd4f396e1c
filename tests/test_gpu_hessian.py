"""xtb_hessian through the C ABI: the displaced single points run on the batched engine.

The reference's own C test (c_api_example.c:242-261) checks three Hessian elements of the
propyne test molecule at 1e-9; the oracle's Hessian (same displacements, same start
wavefunction) is the check for every element, and for the dipole gradient.
"""
import numpy as np
import pytest

from helpers import case_geometry, golden
from oracle import gfn2
from xtb_gb300 import interface as X
from xtb_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_hessian_matches_reference_c_api_values():
    case = golden()["capi_hessian"]
    Z, xyz = case_geometry(case)
    H, _ = X.Calculator(Z, xyz).hessian()
    flat = H.T.ravel()
    for c in case["checks"]:
        i = int(c["expr"][5:-1])
        assert abs(flat[i] - c["value"]) <= c["thr"], (c["expr"], flat[i], c["value"])
    assert abs(flat[3] - flat[63]) <= 1e-9
    assert np.array_equal(H, H.T)


def test_hessian_and_dipole_gradient_match_oracle():
    Z, xyz = W.alkane(3, 0.02, seed=4)            # propane, 11 atoms: 66 displaced single points
    H, dg = X.Calculator(Z, xyz).hessian()
    Ho, dgo = gfn2.hessian(Z, xyz)
    assert np.max(np.abs(H - Ho)) <= 1e-6
    assert np.max(np.abs(dg - dgo)) <= 1e-6
    # translational invariance: rows sum to ~0 over each Cartesian direction
    n = len(Z)
    for c in range(3):
        assert np.max(np.abs(H[:, c::3].sum(axis=1))) <= 1e-5


def test_hessian_rejects_unsupported_arguments():
    Z, xyz = W.alkane(1, 0.02, seed=1)
    calc = X.Calculator(Z, xyz)
    import ctypes as C
    n3 = 3 * len(Z)
    hess = np.zeros((n3, n3))
    pol = np.zeros((n3, 6))
    calc.lib.xtb_hessian(calc.env.h, calc.mol, calc.calc, calc.res, hess.ctypes.data_as(C.POINTER(C.c_double)),
                         None, None, None, pol.ctypes.data_as(C.POINTER(C.c_double)))
    with pytest.raises(X.XTBException, match="Polarizability"):
        calc.env.check()


def test_virial_is_the_strain_derivative():
    """xtb_getVirial = dE/d(strain): central differences of the energy under homogeneous strain."""
    import ctypes as C
    Z, xyz = W.water_cluster(3, seed=2)
    calc = X.Calculator(Z, xyz)
    calc.singlepoint()
    sig = np.zeros(9)
    calc.lib.xtb_getVirial(calc.env.h, calc.res, sig.ctypes.data_as(C.POINTER(C.c_double)))
    calc.env.check()
    sig = sig.reshape(3, 3)
    h = 1e-4
    fd = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            e = []
            for s in (1.0, -1.0):
                eps = np.eye(3)
                eps[i, j] += s * h
                e.append(X.Calculator(Z, xyz @ eps.T).singlepoint().energy)
            fd[i, j] = (e[0] - e[1]) / (2 * h)
    assert np.max(np.abs(fd - sig)) <= 1e-6, (fd, sig)
