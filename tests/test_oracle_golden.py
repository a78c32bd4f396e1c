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


def _solvation(Z, case):
    from oracle import solvation as S
    from oracle.params import AATOAU
    if "model" in case:
        return S.Solvation(Z, case["solvent"], model=case["model"])
    return S.Solvation(Z, case["solvent"], kernel=case["kernel"], alpb=case["alpb"],
                       ion_strength=case.get("ion_strength", 0.0),
                       ion_rad=case.get("ion_rad_angstrom", 0.0) * AATOAU)


@pytest.mark.parametrize("key", ["gbsa", "salt"])
def test_oracle_implicit_solvation(key):
    """test_gfn2.f90:237-381: GBSA in water and salt-screened GBSA in CH2Cl2, each from the EEQ
    guess: energy, gap, gradient norm and components."""
    case = CASES[key]
    Z, xyz = case_geometry(case)
    r = gfn2.singlepoint(Z, xyz, maxiter=case["maxiter"], solvation=_solvation(Z, case))
    assert r.converged
    for c in case["checks"]:
        got = evaluate(c["expr"], r)
        assert abs(got - c["value"]) <= c["thr"], (c["expr"], got, c["value"], c["thr"])


def test_oracle_c_api_solvation_chain():
    """c_api_example.c:38-163: propyne in vacuum, then xtb_setSolvent "gbsa" and "alpb" in water,
    each single point started from the previous result: energy, q[5], dipole[2], wbo[9]."""
    case = CASES["capi"]
    Z, xyz = case_geometry(case)
    prev = gfn2.singlepoint(Z, xyz, maxiter=case["maxiter"])
    for key in ("capi_gbsa", "capi_alpb"):
        c2 = CASES[key]
        r = gfn2.singlepoint(Z, xyz, maxiter=c2["maxiter"], solvation=_solvation(Z, c2), q_init=prev.q,
                             qsh_init=prev.qsh, dipm_init=prev.dipm, qp_init=prev.qp)
        assert r.converged
        for c in c2["checks"]:
            got = evaluate(c["expr"], r)
            assert abs(got - c["value"]) <= c["thr"], (key, c["expr"], got, c["value"], c["thr"])
        prev = r


def test_oracle_mindless_solvation():
    """test_gfn2.f90:745-828: mindless01-10 in ten solvents (GBSA parameters, Still kernel, the
    ALPB shape correction on every second molecule): energy, gradient norm and gap at 1e-8."""
    for m in CASES["mindless_solvation"]:
        Z = np.array(m["numbers"])
        xyz = np.array(m["positions"], dtype=float).reshape(-1, 3)
        r = gfn2.singlepoint(Z, xyz, solvation=_solvation(Z, m))
        assert abs(r.energy - m["energy"]) <= m["thr"], m["name"]
        assert abs(np.linalg.norm(r.gradient) - m["gnorm"]) <= m["thr"], m["name"]
        assert abs(r.hl_gap - m["hl_gap"]) <= m["thr"], m["name"]


def test_oracle_solvation_gradient_matches_finite_difference():
    """The solvation gradient (Born radii chain, SASA, H-bond, ALPB shape term) of a charged
    molecule against central differences of the solvation energy at fixed charges.

    The salt-screened kernel's gradient is the reference's (src/solv/kernel.f90, the self term of
    addGradientSaltStill), whose Born-radius derivative of the self energy carries
    discr + ionscr*kappa where the exact derivative has discr - ionscr*kappa; it is restated as it
    is (the reference's salt test pins it) and checked here at the size of that difference."""
    from oracle import solvation as S
    case = CASES["capi"]
    Z, xyz = case_geometry(case)
    q = np.array([0.3, -0.2, 0.1, 0.25, -0.15, 0.2, 0.3])             # net charge 0.8
    for kw, tol in (({"model": "gbsa"}, 1e-8), ({"model": "alpb"}, 1e-8), ({"kernel": "still", "alpb": True}, 1e-8),
                    ({"kernel": "still", "alpb": False, "ion_strength": 1e-3, "ion_rad": 1.9}, 2e-7)):
        sv = S.Solvation(Z, "water", **kw)
        g = sv.update(xyz).gradient(q)
        h = 1e-5
        for a in (0, 3, 6):
            for k in range(3):
                xp, xm = xyz.copy(), xyz.copy()
                xp[a, k] += h
                xm[a, k] -= h
                fd = (sv.update(xp).energy(q) - sv.update(xm).energy(q)) / (2 * h)
                assert abs(fd - g[a, k]) < tol, (kw, a, k, fd, g[a, k])
