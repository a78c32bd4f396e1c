"""GPU parity of the plain FP64 engine through the C ABI (needs a GB300).

Tolerances (stated once, used everywhere): |dE| <= 1e-6 Eh, charges <= 1e-5 e,
gradient components <= 1e-5 Eh/bohr, SCC iterations within +-1 of the oracle.
"""
import os
import subprocess
import types

import numpy as np
import pytest

from helpers import TOL_E, TOL_G, TOL_ITER, TOL_Q, case_geometry, evaluate, golden
from oracle import gfn2
from oracle.params import EVTOAU
from xtb_gb300 import interface as X
from xtb_gb300 import workloads as W

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def gpu(Z, xyz, **kw):
    return X.Calculator(Z, xyz, **kw).singlepoint()


def as_eval(r):
    return types.SimpleNamespace(energy=r.energy, gnorm=r.gnorm, hl_gap=r.hl_gap, gradient=r.gradient,
                                 q=r.charges, dipole=r.dipole, wbo=r.bond_orders)


def assert_parity(r, o, iters=True):
    assert abs(r.energy - o.energy) <= TOL_E, (r.energy, o.energy)
    assert np.max(np.abs(r.charges - o.q)) <= TOL_Q
    assert np.max(np.abs(r.gradient - o.gradient)) <= TOL_G
    if iters:
        assert abs(r.iterations - o.iterations) <= TOL_ITER, (r.iterations, o.iterations)


@pytest.mark.parametrize("key", ["api", "pcem", "capi"])
def test_reference_known_answers(key):
    """Values asserted by the reference's own tests, reproduced through the C ABI."""
    case = golden()[key]
    Z, xyz = case_geometry(case)
    r = gpu(Z, xyz, maxiter=case["maxiter"])
    assert r.converged
    e = as_eval(r)
    for c in case["checks"]:
        kind = "g" if "gradient" in c["expr"] else ("q" if c["expr"].startswith("q") else "e")
        tol = min({"e": TOL_E, "g": TOL_G, "q": TOL_Q}[kind] if kind != "e" or "gap" not in c["expr"] else 1e-4,
                  max(c["thr"], 2e-10))
        got = evaluate(c["expr"], e)
        assert abs(got - c["value"]) <= tol, (c["expr"], got, c["value"], tol)


MOLECULES = {
    "water": ([8, 1, 1], [[0.0, 0.0, -0.7357858611], [1.4418315287, 0.0, 0.3678929305], [-1.4418315287, 0.0, 0.3678929305]], 0, 0),
    "hydroxide": ([8, 1], [[0.0, 0.0, 0.0], [0.0, 0.0, 1.83]], -1, 0),
    "ammonium": ([7, 1, 1, 1, 1], [[0, 0, 0], [1.12, 1.12, 1.12], [-1.12, -1.12, 1.12], [-1.12, 1.12, -1.12], [1.12, -1.12, -1.12]], 1, 0),
    "methyl_radical": ([6, 1, 1, 1], [[0, 0, 0], [2.04, 0, 0], [-1.02, 1.767, 0], [-1.02, -1.767, 0.05]], 0, 1),
    "hydrogen_sulfide": ([16, 1, 1], [[0, 0, 0], [2.52, 0, 0.1], [-0.2, 2.5, 0]], 0, 0),
    "silane": ([14, 1, 1, 1, 1], [[0, 0, 0], [1.61, 1.61, 1.61], [-1.61, -1.61, 1.61], [-1.61, 1.61, -1.61], [1.61, -1.61, -1.6]], 0, 0),
    "hydrogen_chloride": ([17, 1], [[0, 0, 0], [0, 0, 2.41]], 0, 0),
    "dihydrogen": ([1, 1], [[0, 0, 0], [0, 0, 1.4]], 0, 0),
}


@pytest.mark.parametrize("name", sorted(MOLECULES))
def test_small_molecules_match_oracle(name):
    Z, xyz, charge, uhf = MOLECULES[name]
    xyz = np.array(xyz, dtype=float)
    r = gpu(Z, xyz, charge=charge, uhf=uhf)
    o = gfn2.singlepoint(Z, xyz, charge=charge, uhf=uhf)
    assert_parity(r, o)


@pytest.mark.parametrize("n", [1, 2, 3, 7])
def test_alkanes_match_oracle(n):
    Z, xyz = W.alkane(n, 0.02, seed=10 + n)
    assert_parity(gpu(Z, xyz), gfn2.singlepoint(Z, xyz))


@pytest.mark.parametrize("m", [2, 5, 12])
def test_water_clusters_match_oracle(m):
    Z, xyz = W.water_cluster(m, seed=20 + m)
    assert_parity(gpu(Z, xyz), gfn2.singlepoint(Z, xyz))


@pytest.mark.parametrize("name", ["c10h22_seed1", "h2o_30_seed1", "c50h102_seed3", "h2o_300_seed1", "c200h402_seed1"])
def test_workload_fixtures(name):
    path = os.path.join(GOLD, f"{name}.npz")
    if not os.path.exists(path):
        pytest.skip(f"fixture {name} not generated")
    f = np.load(path)
    r = gpu(f["numbers"], f["positions"])
    o = types.SimpleNamespace(energy=float(f["energy"]), q=f["charges"], gradient=f["gradient"],
                              iterations=int(f["iterations"]))
    assert_parity(r, o)


def test_full_size_invariants():
    """(H2O)300 (N = 900, nao = 1800): charge conservation, zero net force, and the
    gradient against a central finite difference of the energy along a random direction."""
    Z, xyz = W.water_cluster(300, seed=1)
    calc = X.Calculator(Z, xyz)
    r = calc.singlepoint()
    assert abs(np.sum(r.charges)) < 1e-8
    assert np.max(np.abs(np.sum(r.gradient, axis=0))) < 1e-7
    d = np.random.default_rng(5).normal(size=xyz.shape)
    d /= np.linalg.norm(d)
    h = 1e-3
    calc.update(xyz + h * d)
    ep = calc.singlepoint().energy
    calc.update(xyz - h * d)
    em = calc.singlepoint().energy
    fd = (ep - em) / (2 * h)
    assert abs(fd - np.sum(r.gradient * d)) < 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("etemp", [5000.0, 20000.0])
def test_smearing_beyond_the_first_levels(etemp):
    """Inside the SCC the engine bisects the lowest nocc + 32 levels first; at high electronic
    temperature the occupations reach past them, the device gate bisects the rest and the
    smearing runs again: the single point still matches the oracle, orbital energies included."""
    Z, xyz = W.water_cluster(20, seed=2)
    Z, xyz = np.asarray(Z), np.asarray(xyz)
    r = X.Calculator(Z, xyz, etemp=etemp).singlepoint()
    o = gfn2.singlepoint(Z, xyz, etemp=etemp)
    assert r.converged and o.converged
    assert abs(r.energy - o.energy) < TOL_E * 1e-2
    assert np.max(np.abs(r.charges - o.q)) < TOL_Q * 1e-2
    assert np.max(np.abs(r.gradient - o.gradient)) < TOL_G * 1e-3
    assert abs(r.iterations - o.iterations) <= TOL_ITER
    assert np.max(np.abs(r.emo - o.emo * EVTOAU)) < 1e-9     # Hartree against the oracle's eV


def test_warm_start_and_determinism():
    Z, xyz = W.alkane(6, 0.02, seed=3)
    calc = X.Calculator(Z, xyz)
    r1 = calc.singlepoint()
    r2 = calc.singlepoint(fresh=False)               # restarts from the converged charges
    assert abs(r1.energy - r2.energy) < 1e-8
    assert r2.iterations <= r1.iterations
    r3 = calc.singlepoint()
    assert r3.energy == r1.energy                     # bit-identical repeat
    assert np.max(np.abs(r3.gradient - r1.gradient)) < 1e-12


def test_unconverged_scc_reports_error():
    Z, xyz = W.water_cluster(4, seed=2)
    with pytest.raises(X.XTBException, match="did not converge"):
        gpu(Z, xyz, maxiter=2)


def test_c_program_drop_in(tmp_path):
    exe = tmp_path / "test_c_api"
    cmd = ["gcc", "-O1", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "c", "test_c_api.c"),
           "-o", str(exe), "-L", os.path.join(ROOT, "xtb_gb300"), "-lxtb_gb300", "-lm",
           "-Wl,-rpath," + os.path.join(ROOT, "xtb_gb300")]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr


def test_mindless_molecules_reference_values():
    """test_gfn2.f90:667-742 (mindless01-10, many elements) through the C ABI and, all ten at
    once, through the batched engine; the reference checks energy, gradient norm and gap at 1e-8."""
    cases = golden()["mindless"]
    mols = [(np.array(m["numbers"]), np.array(m["positions"], dtype=float).reshape(-1, 3)) for m in cases]
    b = X.Batch(mols).run()
    for i, m in enumerate(cases):
        r = gpu(*mols[i])
        for e, g, gap in ((r.energy, r.gnorm, r.hl_gap), (b.energy[i], np.linalg.norm(b.gradients[i]), b.parts[i, 7])):
            assert abs(e - m["energy"]) <= m["thr"], (m["name"], e, m["energy"])
            assert abs(g - m["gnorm"]) <= m["thr"], (m["name"], g, m["gnorm"])
            assert abs(gap - m["hl_gap"]) <= m["thr"], (m["name"], gap, m["hl_gap"])


def test_fast_reciprocal_within_one_ulp():
    """The reciprocal on the inverse-iteration chains (FP32 seed + one third-order Newton step)
    against the FP64 division, over 6e8 values on both sides of the FP32 seed's range."""
    import ctypes as C
    lib = X.load_library()
    out = np.zeros(2)
    assert lib.xtbgb_reciprocalCheck(out.ctypes.data_as(C.POINTER(C.c_double))) == 0
    assert out[1] == 2001 * 2 * 256 * 586
    assert out[0] <= 1.0, out


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_blocked_backtransform(precision):
    """The compact-WY back-transformation (blocks of 128 reflectors, all T factors in one launch)
    forced below its default 3000-AO threshold: (H2O)50 has 300 AOs, so three blocks, the last
    partial.  It must agree with the warp-per-vector form and with the oracle; with orbitals
    kept, every eigenvector goes through it."""
    Z, xyz = W.water_cluster(50, seed=8)
    base = gpu(Z, xyz, keep_orbitals=False, precision=precision)
    # FP64: both forms are FP64 products in a different order.  Split precision: the two forms
    # feed differently shaped split products (about 2^-40 relative error per product term).
    tol_e, tol = (1e-10, 1e-9) if precision == "fp64" else (1e-8, 1e-8)
    for keep in (False, True):
        r = gpu(Z, xyz, keep_orbitals=keep, precision=precision, blocked_min=0)
        assert abs(r.energy - base.energy) <= tol_e, (r.energy - base.energy)
        assert np.max(np.abs(r.charges - base.charges)) <= tol
        assert np.max(np.abs(r.gradient - base.gradient)) <= tol
        assert r.iterations == base.iterations
    assert_parity(r, gfn2.singlepoint(Z, xyz))


def test_concurrent_threads_match_sequential():
    """Single points on several host threads at once (each thread has its own engine stream and
    workspace) give the sequential results.  The molecules differ in size, so the launches of one
    kernel ask for different dynamic shared-memory sizes at the same time (above 48 KB from 1536
    AOs): the per-kernel limit is process-wide and must never be lowered under another thread."""
    import threading
    mols = [W.water_cluster(270, seed=31), W.water_cluster(40, seed=32), W.alkane(270, 0.02, seed=33),
            W.water_cluster(12, seed=34)]
    seq = [gpu(Z, xyz, keep_orbitals=False) for Z, xyz in mols]
    out = [[None] * len(mols) for _ in range(2)]
    errs = []

    def work(slot, order):
        try:
            for i in order:
                Z, xyz = mols[i]
                out[slot][i] = gpu(Z, xyz, keep_orbitals=False)
        except Exception as e:          # re-raised below on the test's thread
            errs.append(e)

    threads = [threading.Thread(target=work, args=(0, [0, 1, 2, 3])),
               threading.Thread(target=work, args=(1, [2, 3, 0, 1]))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errs, errs
    for slot in range(2):
        for r, s in zip(out[slot], seq):
            assert abs(r.energy - s.energy) <= 1e-9
            assert np.max(np.abs(r.gradient - s.gradient)) <= 1e-9
            assert r.iterations == s.iterations
