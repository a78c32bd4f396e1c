"""The autotuner (needs a GB300).

Its choices only select between kernel forms that compute the same single point, so the
results must not depend on them: a molecule whose size sits where the forms cross over gives
the same energy, charges and gradient with every form pinned (to the rounding of the
different summation orders), and the request loop gives the same results under every schedule.
"""
import numpy as np
import pytest

from xtb_gb300 import interface as X
from xtb_gb300 import tuning
from xtb_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_kernel_forms_measured_and_kept():
    t = tuning.kernel_forms()
    assert t["seconds"] > 0.0
    assert len(t["sytrd_ms"]) >= 5 and len(t["backtransform_ms"]) >= 4
    for row in t["sytrd_ms"]:
        assert row["row_form"] > 0.0 and row["upper_triangle_form"] > 0.0
    g = X.get_tuning()
    assert g["measured"]
    assert (g["sytrd_sym_min"], g["blocked_min_fp64"], g["blocked_min_split"]) == \
        (t["sytrd_sym_min"], t["blocked_min_fp64"], t["blocked_min_split"])
    assert tuning.kernel_forms()["seconds"] == t["seconds"]      # kept, not measured again


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_results_do_not_depend_on_the_forms(precision):
    Z, xyz = W.water_cluster(110, seed=3)             # 660 AOs
    saved = X.get_tuning()
    try:
        X.set_tuning(3, 0, 0)                          # upper-triangle form, blocked back-transformation
        a = X.Calculator(Z, xyz, keep_orbitals=False, precision=precision).singlepoint()
        X.set_tuning(1 << 30, 1 << 30, 1 << 30)        # row form, one warp per vector
        b = X.Calculator(Z, xyz, keep_orbitals=False, precision=precision).singlepoint()
    finally:
        X.set_tuning(saved["sytrd_sym_min"], saved["blocked_min_fp64"], saved["blocked_min_split"])
    assert a.iterations == b.iterations
    assert abs(a.energy - b.energy) <= 1e-9
    assert np.max(np.abs(a.charges - b.charges)) <= 1e-8
    assert np.max(np.abs(a.gradient - b.gradient)) <= 1e-8


@pytest.mark.parametrize("name", ["h3+", "water", "ammonia", "methane", "ethane", "water6", "decane"])
def test_small_matrices_in_both_forms(name):
    """The upper-triangle tridiagonalisation on matrices of 3 to 62 AOs (one tile, a partial
    first row block, more blocks than tiles) against the row form."""
    mols = {
        "h3+": ([1, 1, 1], [[0.0, 0.0, 0.0], [0.0, 0.0, 1.65], [0.0, 1.43, 0.83]], 1),
        "water": ([8, 1, 1], [[0.0, 0.0, 0.0], [0.0, 1.43, 1.1], [0.0, -1.43, 1.1]], 0),
        "ammonia": ([7, 1, 1, 1], [[0.0, 0.0, 0.0], [0.0, 1.77, 0.72], [1.53, -0.89, 0.72], [-1.53, -0.89, 0.72]], 0),
        "methane": ([6, 1, 1, 1, 1], [[0, 0, 0], [1.19, 1.19, 1.19], [-1.19, -1.19, 1.19], [-1.19, 1.19, -1.19],
                                      [1.19, -1.19, -1.19]], 0),
    }
    if name in mols:
        Z, xyz, charge = mols[name]
        Z, xyz = np.array(Z), np.array(xyz, dtype=float)
    else:
        Z, xyz = {"ethane": W.alkane(2, 0.02, seed=1), "water6": W.water_cluster(6, seed=1),
                  "decane": W.alkane(10, 0.02, seed=1)}[name]
        charge = 0
    saved = X.get_tuning()
    try:
        X.set_tuning(3, saved["blocked_min_fp64"], saved["blocked_min_split"])
        a = X.Calculator(Z, xyz, charge=charge).singlepoint()
        X.set_tuning(1 << 30, saved["blocked_min_fp64"], saved["blocked_min_split"])
        b = X.Calculator(Z, xyz, charge=charge).singlepoint()
    finally:
        X.set_tuning(saved["sytrd_sym_min"], saved["blocked_min_fp64"], saved["blocked_min_split"])
    assert a.converged and b.converged and a.iterations == b.iterations
    assert abs(a.energy - b.energy) <= 1e-10
    assert np.max(np.abs(a.charges - b.charges)) <= 1e-9
    assert np.max(np.abs(a.gradient - b.gradient)) <= 1e-9
    assert np.max(np.abs(a.emo - b.emo)) <= 1e-10


def test_wide_tiles_match_the_row_form():
    """From 1800 AOs the upper-triangle tridiagonalisation runs tiles of 16 x 64 (two columns per
    lane) with 16 warps per block: (H2O)683, 4098 AOs, in split mode, against the row form."""
    Z, xyz = W.water_cluster(683, seed=5)
    saved = X.get_tuning()
    try:
        X.set_tuning(3, saved["blocked_min_fp64"], saved["blocked_min_split"])
        a = X.Calculator(Z, xyz, keep_orbitals=False, precision="split").singlepoint()
        X.set_tuning(1 << 30, saved["blocked_min_fp64"], saved["blocked_min_split"])
        b = X.Calculator(Z, xyz, keep_orbitals=False, precision="split").singlepoint()
    finally:
        X.set_tuning(saved["sytrd_sym_min"], saved["blocked_min_fp64"], saved["blocked_min_split"])
    assert a.nao == 4098 and a.converged and b.converged
    assert a.iterations == b.iterations
    assert abs(a.energy - b.energy) <= 1e-8
    assert np.max(np.abs(a.charges - b.charges)) <= 1e-7
    assert np.max(np.abs(a.gradient - b.gradient)) <= 1e-7


def test_schedule_choice_and_results():
    """The schedule tuner picks one of its candidates, and the results do not depend on the
    schedule: worker count, pool step, which molecules the pool takes (here up to 400 AOs or only
    up to 64, the rest on the plain engine) and the cap of the workers' cooperative grids."""
    reqs = W.served_stream(12, seed=5, nmax=400)
    cands = ((2, 1, 512, 0), (4, 2, 64, 24))
    s = tuning.schedule(reqs, candidates=cands, pool_gib=2.0, max_slots=64)
    assert (s["plain_workers"], s["iters_per_step"], s["pool_max_nao"], s["coop_blocks"]) in cands
    assert len(s["span_s"]) == 2
    out = {}
    for w, i, p, cb in cands:
        srv = X.Server(pool_gib=2.0, max_slots=64, plain_workers=w, iters_per_step=i, pool_max_nao=p, coop_blocks=cb)
        out[w] = [srv.wait(srv.submit(r["numbers"], r["positions"], gradient=r["gradient"])) for r in reqs]
        srv.close()
    assert sum(x.engine for x in out[4]) > sum(x.engine for x in out[2])    # more on the plain engine
    for r2, r4 in zip(out[2], out[4]):
        assert abs(r2.energy - r4.energy) <= 1e-9


def test_capped_cooperative_tridiagonalisation():
    """Both tridiagonalisation forms with a capped grid (16 and 40 blocks, and one block per 20
    AOs of the request) give the single point of the full grid: the request loop with every
    molecule on the workers against the plain calculator."""
    reqs = W.served_stream(6, seed=9, nmin=40, nmax=300)
    saved = X.get_tuning()
    try:
        for sym in (1 << 30, 3):                           # row form, upper-triangle form
            X.set_tuning(sym, saved["blocked_min_fp64"], saved["blocked_min_split"])
            ref = [X.Calculator(r["numbers"], r["positions"], keep_orbitals=False).singlepoint() for r in reqs]
            for cap in (16, 40, -20):
                srv = X.Server(pool_gib=1.0, max_slots=8, plain_workers=2, pool_max_nao=1, coop_blocks=cap)
                out = [srv.wait(srv.submit(r["numbers"], r["positions"], gradient=r["gradient"])) for r in reqs]
                srv.close()
                for a, b in zip(out, ref):
                    assert a.engine == 1
                    assert abs(a.energy - b.energy) <= 1e-9, (sym, cap)
    finally:
        X.set_tuning(saved["sytrd_sym_min"], saved["blocked_min_fp64"], saved["blocked_min_split"])


def test_sytrd_timing_entry_point():
    """xtbgb_sytrdMs times one tridiagonalisation with a chosen form and grid cap and refuses
    sizes and forms outside its range."""
    for form, cap in ((0, 0), (1, 0), (1, 38), (-1, 0)):
        assert X.sytrd_ms(300, form, cap, 1) > 0.0
    for n, form in ((2, 1), (9000, 1), (300, 2)):
        with pytest.raises(X.XTBException):
            X.sytrd_ms(n, form, 0, 1)


@pytest.mark.parametrize("n,ncol", [(5, 3), (300, 300), (700, 7), (1000, 1000), (1800, 1200), (2600, 2600)])
def test_fp64_strip_backtransformation(n, ncol):
    """The FP64 compact-WY back-transformation (one launch, a strip of columns per block) against
    one warp per vector: strips of 1 to 16 columns, idle blocks (7 columns over all SMs), and
    strips wider than one pass (2600 columns)."""
    err, ms_warp, ms_strips = X.backtransform_check(n, ncol, 0)
    assert err <= 1e-12, (n, ncol, err)
    assert ms_warp > 0.0 and ms_strips > 0.0


def test_split_backtransformation_check():
    err, _, _ = X.backtransform_check(1200, 600, 5)
    assert err <= 1e-9
    for n, ncol, slices in ((2, 1, 0), (300, 0, 0), (300, 301, 0), (300, 10, 9)):
        with pytest.raises(X.XTBException):
            X.backtransform_check(n, ncol, slices)
