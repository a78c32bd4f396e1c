"""The CPU oracle against the reference's own known-answer tests (CPU only).

Pins the oracle: every value the reference's GFN2 tests assert
(test/unit/test_gfn2.f90 scc/api/pcem, test/api/c_api_example.c) must be
reproduced at the tolerance the reference asserts it at.
"""
import numpy as np
import pytest

from helpers import case_geometry, evaluate, golden
from oracle import gfn2

CASES = golden()


@pytest.mark.parametrize("key", ["scc", "api", "pcem", "capi"])
def test_oracle_reproduces_reference(key):
    case = CASES[key]
    Z, xyz = case_geometry(case)
    r = gfn2.singlepoint(Z, xyz, maxiter=case["maxiter"], guess=case["guess"])
    assert r.converged
    for c in case["checks"]:
        got = evaluate(c["expr"], r)
        assert abs(got - c["value"]) <= c["thr"] + 1e-12, (c["expr"], got, c["value"], c["thr"])


def test_oracle_translation_invariance():
    case = CASES["api"]
    Z, xyz = case_geometry(case)
    r0 = gfn2.singlepoint(Z, xyz)
    r1 = gfn2.singlepoint(Z, xyz + np.array([3.0, -2.0, 7.5]))
    # moments are taken about the coordinate origin (as in the reference), so a shift
    # costs a few digits through cancellation; the bound is far below the parity tolerance
    assert abs(r0.energy - r1.energy) < 1e-8
    assert np.max(np.abs(r0.gradient - r1.gradient)) < 1e-8


def test_oracle_gradient_matches_finite_difference():
    case = CASES["api"]
    Z, xyz = case_geometry(case)
    g = gfn2.singlepoint(Z, xyz).gradient
    h = 1e-4
    for (a, k) in [(0, 2), (3, 0), (6, 2)]:
        xp, xm = xyz.copy(), xyz.copy()
        xp[a, k] += h
        xm[a, k] -= h
        fd = (gfn2.singlepoint(Z, xp).energy - gfn2.singlepoint(Z, xm).energy) / (2 * h)
        assert abs(fd - g[a, k]) < 2e-6, (a, k, fd, g[a, k])


def test_oracle_hessian_matches_reference_c_api_test():
    """c_api_example.c:242-261: numerical Hessian of the propyne test molecule, fresh results
    object, default step; the reference checks three elements at 1e-9."""
    case = golden()["capi_hessian"]
    Z, xyz = case_geometry(case)
    H, _ = gfn2.hessian(Z, xyz, step=case["step"])
    flat = H.T.ravel()                       # column-major, as the C array
    for c in case["checks"]:
        i = int(c["expr"][5:-1])
        assert abs(flat[i] - c["value"]) <= c["thr"], (c["expr"], flat[i], c["value"])
    assert np.max(np.abs(H - H.T)) == 0.0


def test_oracle_mindless_molecules():
    """test_gfn2.f90:667-742: ten random 16-atom molecules over many elements (mindless01-10,
    geometries of test/unit/molstock.f90), energy, gradient norm and gap at 1e-8."""
    for m in golden()["mindless"]:
        Z = np.array(m["numbers"])
        xyz = np.array(m["positions"], dtype=float).reshape(-1, 3)
        r = gfn2.singlepoint(Z, xyz)
        assert abs(r.energy - m["energy"]) <= m["thr"], m["name"]
        assert abs(np.linalg.norm(r.gradient) - m["gnorm"]) <= m["thr"], m["name"]
        assert abs(r.hl_gap - m["hl_gap"]) <= m["thr"], m["name"]


@pytest.mark.parametrize("key", ["pcem_charges", "pcem_point", "capi_pc"])
def test_oracle_external_point_charges(key):
    """test_gfn2.f90:459-520 (water dimer in the field of six charges, GFN2 hardnesses and
    gamma = 999) and c_api_example.c:298-410 (the same through xtb_setExternalCharges, which
    takes each charge's hardness from its element): energy, gradient, point-charge gradient."""
    from oracle.params import get_params
    case = CASES[key]
    Z, xyz = case_geometry(case)
    gam = case.get("pc_gam") or [get_params().chemicalHardness[z - 1] for z in case["pc_numbers"]]
    r = gfn2.singlepoint(Z, xyz, maxiter=case["maxiter"], pc_charges=case["pc_charges"],
                         pc_positions=case["pc_positions"], pc_gam=gam)
    assert r.converged
    for c in case["checks"]:
        got = evaluate(c["expr"], r)
        assert abs(got - c["value"]) <= c["thr"], (c["expr"], got, c["value"], c["thr"])
