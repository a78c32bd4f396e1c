"""Implicit-solvent host logic (CPU only): the Lebedev-Laikov tables, solvent resolution and the
errors xtb_setSolvent pushes (src/api/calculator.f90:341-439, src/solv/model.f90)."""
import numpy as np
import pytest

from helpers import case_geometry, golden
from oracle import solvation as S
from xtb_gb300 import interface as X


@pytest.mark.parametrize("size", S.data()["lebedev_sizes"])
def test_lebedev_grids_integrate_polynomials(size):
    """Every extracted grid expands to its size, lies on the unit sphere and integrates the
    monomials x^2, x^4, x^2 y^2 exactly (weights normalised to 1)."""
    pts, w = S.lebedev_grid(size if size != S.data()["lebedev_sizes"][-1] else size + 1)
    assert len(pts) == size
    assert np.max(np.abs(np.sum(pts ** 2, axis=1) - 1.0)) < 1e-14
    assert abs(w.sum() - 1.0) < 1e-13
    assert abs(np.sum(w * pts[:, 0] ** 2) - 1.0 / 3.0) < 1e-13
    if size >= 14:
        assert abs(np.sum(w * pts[:, 0] ** 4) - 1.0 / 5.0) < 1e-13
        assert abs(np.sum(w * pts[:, 0] ** 2 * pts[:, 1] ** 2) - 1.0 / 15.0) < 1e-13


def test_grid_selection_follows_the_reference_bisection():
    sizes = S.data()["lebedev_sizes"]
    assert len(S.lebedev_grid(230)[1]) == 230
    assert len(S.lebedev_grid(231)[1]) == 230
    assert len(S.lebedev_grid(sizes[-1])[1]) == sizes[-2]      # x == last size selects the one below
    assert len(S.lebedev_grid(10 ** 6)[1]) == sizes[-1]
    with pytest.raises(ValueError):
        S.lebedev_grid(5)


def test_parameter_sets_and_aliases():
    assert S.parameter_set("water", "still") is S.parameter_set("h2o", "still")
    assert S.parameter_set("H2O", "p16") is S.data()["alpb"]["water"]
    assert S.parameter_set("n-hexane", "still") is S.data()["gbsa"]["nhexan"]
    assert S.parameter_set("chloroform", "p16") is S.data()["alpb"]["chcl3"]
    with pytest.raises(KeyError):
        S.parameter_set("furane", "still")          # an ALPB-only solvent


@pytest.fixture()
def calc():
    try:
        X.load_library()
    except X.XTBException as e:
        pytest.skip(str(e))
    Z, xyz = case_geometry(golden()["capi"])
    return X.Calculator(Z, xyz)


def test_set_solvent_errors(calc):
    for solvent, model, text in (("unobtainium", "gbsa", "not parametrized"), ("furane", "gbsa", "not parametrized"),
                                 ("water", "cosmo", "not supported"), ("water", "cpcmx", "not supported"),
                                 ("water", "pcm", "Unknown solvation model")):
        with pytest.raises(X.XTBException, match=text):
            calc.set_solvent(solvent, model)
    with pytest.raises(X.XTBException, match="Invalid angular grid"):
        calc.set_solvent("water", "gbsa", grid=5)
    calc.set_solvent("furane", "alpb")                      # ALPB has furane
    calc.set_solvent("Methylenechloride", "gbsa", state=2, temperature=310.0, grid=590)
    calc.set_solvent("none")                                # gas phase: no error
    calc.release_solvent()
    with pytest.raises(X.XTBException, match="No solvation model set"):
        calc.lib.xtbgb_setSolventKernel(calc.env.h, calc.calc, 0)
        calc.env.check()
    calc.set_solvent("water", "alpb", ion_strength=1e-3, ion_rad=1.0, kernel="still")
    with pytest.raises(X.XTBException, match="Still"):
        calc.set_solvent("water", "alpb", kernel="p16")
