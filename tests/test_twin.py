"""The C++/OpenMP + LAPACK twin of the oracle (CPU only).

The twin is what the CPU baseline times, so it is pinned the same way the NumPy oracle is:
the reference's own known-answer values (test/unit/test_gfn2.f90 scc/api/pcem, mindless01-10,
test/api/c_api_example.c), the committed oracle fixtures of the benchmark geometries, and the
NumPy oracle itself on an open-shell molecule.
"""
import numpy as np
import pytest

from helpers import case_geometry, evaluate, golden
from oracle import gfn2, twin

CASES = golden()


@pytest.fixture(scope="module", autouse=True)
def built():
    twin.build()


@pytest.mark.parametrize("key", ["scc", "api", "pcem", "capi"])
def test_twin_reproduces_reference(key):
    case = CASES[key]
    Z, xyz = case_geometry(case)
    r = twin.singlepoint(Z, xyz, maxiter=case["maxiter"], guess=case["guess"], wbo=True)
    assert r.converged
    for c in case["checks"]:
        if c["expr"].startswith(("wfn%dipm", "wfn%qp")):
            continue          # the twin returns no atomic multipoles (the NumPy oracle checks them)
        got = evaluate(c["expr"], r)
        assert abs(got - c["value"]) <= c["thr"] + 1e-12, (c["expr"], got, c["value"], c["thr"])


def test_twin_mindless_molecules():
    """test_gfn2.f90:667-742: mindless01-10 (H to heavy main-group elements, s/p/d shells),
    energy, gradient norm and HOMO-LUMO gap at the reference's 1e-8."""
    for m in CASES["mindless"]:
        Z = np.array(m["numbers"])
        xyz = np.array(m["positions"], dtype=float).reshape(-1, 3)
        r = twin.singlepoint(Z, xyz)
        assert abs(r.energy - m["energy"]) <= m["thr"], m["name"]
        assert abs(r.gnorm - m["gnorm"]) <= m["thr"], m["name"]
        assert abs(r.hl_gap - m["hl_gap"]) <= m["thr"], m["name"]


@pytest.mark.parametrize("name", ["c10h22_seed1", "h2o_30_seed1", "c50h102_seed3", "h2o_300_seed1"])
def test_twin_matches_workload_fixtures(name):
    """The committed oracle results of the benchmark geometries (made by
    tests/golden/make_workload_fixtures.py), up to (H2O)300 with 1800 orbitals."""
    d = np.load(f"{__file__.rsplit('/', 1)[0]}/golden/{name}.npz")
    r = twin.singlepoint(d["numbers"], d["positions"])
    assert r.converged
    assert abs(r.energy - float(d["energy"])) <= 1e-9
    assert np.max(np.abs(r.q - d["charges"])) <= 1e-8
    assert np.max(np.abs(r.gradient - d["gradient"])) <= 1e-8
    assert r.iterations == int(d["iterations"])
    assert np.max(np.abs(r.emo - d["emo"])) <= 1e-7


def test_twin_matches_oracle_open_shell_and_dipole():
    """Methyl radical (odd electron count: separate alpha/beta Fermi levels and the
    unrestricted bond orders) against the NumPy oracle, including dipole and bond orders."""
    Z = np.array([6, 1, 1, 1])
    xyz = np.array([[0, 0, 0], [2.04, 0, 0], [-1.02, 1.767, 0], [-1.02, -1.767, 0.05]], dtype=float)
    r = twin.singlepoint(Z, xyz, wbo=True)
    o = gfn2.singlepoint(Z, xyz)
    assert abs(r.energy - o.energy) <= 1e-10
    assert np.max(np.abs(r.gradient - o.gradient)) <= 1e-10
    assert np.max(np.abs(r.q - o.q)) <= 1e-9
    assert np.max(np.abs(r.dipole - o.dipole)) <= 1e-9
    assert np.max(np.abs(r.wbo - o.wbo)) <= 1e-9
    assert r.iterations == o.iterations
