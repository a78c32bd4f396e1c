"""GBSA / ALPB implicit solvation on the GPU against the reference's known answers and the oracle.

Reference cases: test/unit/test_gfn2.f90:237-381 (GBSA in water, salt-screened GBSA in CH2Cl2),
:745-828 (mindless01-10 in ten solvents, ALPB correction on every second one) and
test/api/c_api_example.c:114-163 (propyne through xtb_setSolvent "gbsa" then "alpb", each from
the previous result).  Every single point here runs through the C ABI.
"""
import numpy as np
import pytest

from helpers import TOL_E, TOL_G, TOL_Q, case_geometry, evaluate, golden
from oracle import gfn2
from oracle import solvation as S
from oracle.params import AATOAU
from xtb_gb300 import interface as X
from xtb_gb300 import workloads as W

pytestmark = pytest.mark.gpu
CASES = golden()


def calc_for(Z, xyz, case, **kw):
    c = X.Calculator(Z, xyz, maxiter=case.get("maxiter", 250), **kw)
    c.set_solvent(case["solvent"], "alpb" if case["alpb"] else "gbsa", ion_strength=case.get("ion_strength"),
                  ion_rad=case.get("ion_rad_angstrom", 0.0) * AATOAU, kernel=case["kernel"])
    return c


@pytest.mark.parametrize("key", ["gbsa", "salt"])
def test_reference_solvation_cases(key):
    """GBSA (water) and salt-screened GBSA (CH2Cl2, 1 mM, 1 A ions): the reference's energy,
    gap and gradient values at its tolerances, and the oracle's gradient at 1e-9."""
    case = CASES[key]
    Z, xyz = case_geometry(case)
    r = calc_for(Z, xyz, case).singlepoint()
    assert r.converged and r.solvated
    for c in case["checks"]:
        got = evaluate(c["expr"], r)
        assert abs(got - c["value"]) <= c["thr"], (c["expr"], got, c["value"])
    sv = S.Solvation(Z, case["solvent"], kernel="still", alpb=False, ion_strength=case.get("ion_strength", 0.0),
                     ion_rad=case.get("ion_rad_angstrom", 0.0) * AATOAU)
    o = gfn2.singlepoint(Z, xyz, maxiter=case["maxiter"], solvation=sv)
    assert abs(r.energy - o.energy) < 1e-9
    assert np.max(np.abs(r.gradient - o.gradient)) < 1e-9
    assert abs(r.g_solv - o.e_solv) < 1e-9


def test_c_api_solvation_chain():
    """c_api_example.c:114-163: the vacuum single point, then GBSA and ALPB water, warm-started."""
    case = CASES["capi"]
    Z, xyz = case_geometry(case)
    calc = X.Calculator(Z, xyz, maxiter=30)
    calc.singlepoint()
    for key in ("capi_gbsa", "capi_alpb"):
        c2 = CASES[key]
        calc.release_solvent()
        calc.set_solvent(c2["solvent"], c2["model"])
        r = calc.singlepoint(fresh=False)
        assert r.solvated
        for c in c2["checks"]:
            got = evaluate(c["expr"], r)
            assert abs(got - c["value"]) <= c["thr"], (key, c["expr"], got, c["value"])


def test_mindless_solvation_reference_values():
    """test_gfn2.f90:745-828: energy, gradient norm and gap at 1e-8 in ten solvents, every second
    one with the ALPB correction on the Still kernel (xtbgb_setSolventKernel)."""
    for m in CASES["mindless_solvation"]:
        Z = np.array(m["numbers"])
        xyz = np.array(m["positions"], dtype=float).reshape(-1, 3)
        c = X.Calculator(Z, xyz)
        c.set_solvent(m["solvent"], "alpb" if m["alpb"] else "gbsa", kernel="still")
        r = c.singlepoint()
        assert abs(r.energy - m["energy"]) <= m["thr"], m["name"]
        assert abs(r.gnorm - m["gnorm"]) <= m["thr"], m["name"]
        assert abs(r.hl_gap - m["hl_gap"]) <= m["thr"], m["name"]


@pytest.mark.parametrize("model,charge,uhf", [("gbsa", 0, 0), ("alpb", 0, 0), ("alpb", 1, 1), ("gbsa", -1, 1)])
def test_solvated_ions_and_models_match_oracle(model, charge, uhf):
    """A water cluster with a charge (the ALPB shape term acts only on charged molecules), both
    models, against the oracle: energy, charges, gradient and the solvation parts."""
    Z, xyz = W.water_cluster(12, seed=4)
    Z, xyz = np.asarray(Z), np.asarray(xyz)
    c = X.Calculator(Z, xyz, charge=charge, uhf=uhf)
    c.set_solvent("water", model)
    r = c.singlepoint()
    o = gfn2.singlepoint(Z, xyz, charge=charge, uhf=uhf, solvation=S.Solvation(Z, "water", model))
    assert r.converged and o.converged
    assert abs(r.energy - o.energy) < TOL_E * 1e-2
    assert np.max(np.abs(r.charges - o.q)) < TOL_Q * 1e-2
    assert np.max(np.abs(r.gradient - o.gradient)) < TOL_G * 1e-3
    assert abs(r.g_solv - o.e_solv) < 1e-8
    assert abs(r.iterations - o.iterations) <= 1


def test_solvent_options_and_errors():
    """Solution state shift, temperature and grid size reach the model; unknown solvents and the
    models this engine does not implement push errors; "none" is the gas phase."""
    Z, xyz = case_geometry(CASES["capi"])
    gas = X.Calculator(Z, xyz).singlepoint()
    c = X.Calculator(Z, xyz)
    c.set_solvent("none")
    r = c.singlepoint()
    assert not r.solvated and abs(r.energy - gas.energy) < 1e-12
    for kw in ({"state": 3, "temperature": 310.0}, {"grid": 590}, {"grid": 5810}):
        c = X.Calculator(Z, xyz)
        c.set_solvent("acetonitrile", "alpb", **kw)
        r = c.singlepoint()
        sv = S.Solvation(Z, "acetonitrile", "alpb", nang=kw.get("grid", 230), state=kw.get("state", 1),
                         temperature=kw.get("temperature", 298.15))
        o = gfn2.singlepoint(Z, xyz, solvation=sv)
        assert abs(r.energy - o.energy) < 1e-9, kw
        assert abs(r.g_shift - sv.gshift) < 1e-15, kw
    c = X.Calculator(Z, xyz)
    for solvent, model, text in (("unobtainium", "gbsa", "not parametrized"), ("water", "cosmo", "not supported"),
                                 ("water", "pcm", "Unknown solvation model"), ("furane", "gbsa", "not parametrized")):
        with pytest.raises(X.XTBException, match=text):
            c.set_solvent(solvent, model)


def test_solvated_hessian_matches_oracle():
    """xtb_hessian with a solvent runs its displaced points on the plain engine; against the
    oracle's Hessian of the same displacements and start wavefunction."""
    Z, xyz = case_geometry(CASES["capi"])
    c = X.Calculator(Z, xyz)
    c.set_solvent("water", "alpb")
    H, dg = c.hessian()
    Ho, dgo = gfn2.hessian(Z, xyz, solvation=S.Solvation(Z, "water", "alpb"))
    assert np.max(np.abs(H - Ho)) <= 1e-6
    assert np.max(np.abs(dg - dgo)) <= 1e-6


@pytest.mark.parametrize("Z,xyz", [([10], [[0.0, 0.0, 0.0]]), ([1, 1], [[0.0, 0.0, 0.0], [0.0, 0.0, 1.4]])])
def test_smallest_solutes(Z, xyz):
    """A single atom (empty neighbour lists, one Born radius) and H2 in implicit water."""
    Z, xyz = np.array(Z), np.array(xyz, dtype=float)
    for model in ("gbsa", "alpb"):
        c = X.Calculator(Z, xyz)
        c.set_solvent("water", model)
        r = c.singlepoint()
        o = gfn2.singlepoint(Z, xyz, solvation=S.Solvation(Z, "water", model))
        assert abs(r.energy - o.energy) < 1e-9, model
        assert np.max(np.abs(r.gradient - o.gradient)) < 1e-9, model
        assert abs(r.g_solv - o.e_solv) < 1e-10, model


def test_solvent_with_external_charges():
    """Point charges and an implicit solvent together (the reference adds both to the same SCC):
    the water dimer of the reference's point-charge test in ALPB water."""
    from oracle.params import get_params
    case = CASES["capi_pc"]
    Z, xyz = case_geometry(case)
    gam = [get_params().chemicalHardness[z - 1] for z in case["pc_numbers"]]
    c = X.Calculator(Z, xyz)
    c.set_external_charges(case["pc_charges"], case["pc_positions"], numbers=case["pc_numbers"])
    c.set_solvent("water", "alpb")
    r = c.singlepoint()
    o = gfn2.singlepoint(Z, xyz, pc_charges=case["pc_charges"], pc_positions=case["pc_positions"], pc_gam=gam,
                         solvation=S.Solvation(Z, "water", "alpb"))
    assert abs(r.energy - o.energy) < 1e-9
    assert np.max(np.abs(r.gradient - o.gradient)) < 1e-9
    assert np.max(np.abs(r.pcgrad - o.pcgrad)) < 1e-9
