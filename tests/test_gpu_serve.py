"""Request loop (continuous batching) against the plain engine.

A served result must equal the plain engine's result for the same molecule (the pool
runs the same device arithmetic; only summation orders differ): |dE| <= 1e-9 Eh,
charges and gradient <= 1e-7.  A molecule's result must not depend on what else is in
flight: alone and in the mix agree to 1e-10 Eh (gradient sums use atomics).
"""
import time

import numpy as np
import pytest

from helpers import TOL_ITER
from xtb_gb300 import interface as X
from xtb_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def mixed_requests(seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(24):
        if k % 2 == 0:
            reqs.append(W.alkane(int(rng.integers(1, 15)), 0.02, seed=int(rng.integers(1 << 30))))
        else:
            reqs.append(W.water_cluster(int(rng.integers(2, 25)), seed=int(rng.integers(1 << 30))))
    reqs.append(W.water_cluster(95, seed=5))      # 570 AOs: plain-engine worker
    return reqs


def plain(Z, xyz):
    return X.Calculator(Z, xyz, keep_orbitals=False).singlepoint()


def test_served_results_match_plain_engine():
    reqs = mixed_requests(1)
    srv = X.Server(pool_gib=2.0, max_slots=64, plain_workers=2, iters_per_step=3)
    ids = [srv.submit(Z, xyz) for Z, xyz in reqs]
    res = [srv.wait(i) for i in ids]
    srv.close()
    assert res[-1].engine == 1 and all(r.engine == 0 for r in res[:-1])
    for (Z, xyz), r in zip(reqs, res):
        p = plain(Z, xyz)
        assert r.status == 0 and r.converged == 1
        assert abs(r.energy - p.energy) <= 1e-9, (len(Z), r.energy, p.energy)
        assert np.max(np.abs(r.charges - p.charges)) <= 1e-7
        assert np.max(np.abs(r.gradient - p.gradient)) <= 1e-7
        assert abs(r.iterations - p.iterations) <= TOL_ITER
        assert r.t_submit <= r.t_start <= r.t_done


def test_alone_equals_in_the_mix():
    reqs = mixed_requests(2)
    probe = reqs[7]
    srv = X.Server(pool_gib=2.0, max_slots=64, plain_workers=2, iters_per_step=2)
    alone = srv.wait(srv.submit(*probe))
    # the probe arrives while a full mix is on the GPU
    ids = [srv.submit(Z, xyz) for Z, xyz in reqs[:12]]
    time.sleep(0.05)
    pid = srv.submit(*probe)
    ids += [srv.submit(Z, xyz) for Z, xyz in reqs[12:]]
    mixed = srv.wait(pid)
    for i in ids:
        srv.wait(i)
    srv.close()
    assert abs(alone.energy - mixed.energy) <= 1e-10
    assert np.max(np.abs(alone.charges - mixed.charges)) <= 1e-10
    assert np.max(np.abs(alone.gradient - mixed.gradient)) <= 1e-10
    assert alone.iterations == mixed.iterations


def test_requests_join_while_others_run():
    """Continuous batching: a second wave starts before the first wave has finished."""
    wave_a = [W.water_cluster(m, seed=m) for m in range(10, 30)]
    wave_b = [W.alkane(n, 0.02, seed=n) for n in range(2, 12)]
    srv = X.Server(pool_gib=2.0, max_slots=64, plain_workers=1, iters_per_step=1)
    ida = [srv.submit(Z, xyz) for Z, xyz in wave_a]
    t0 = time.time()
    while srv.stats()["steps"] < 1 and time.time() - t0 < 60:
        time.sleep(0.001)
    idb = [srv.submit(Z, xyz) for Z, xyz in wave_b]
    ra = [srv.wait(i) for i in ida]
    rb = [srv.wait(i) for i in idb]
    srv.close()
    assert min(r.t_start for r in rb) < max(r.t_done for r in ra)
    assert all(r.status == 0 for r in ra + rb)


def test_admission_respects_the_budget():
    """A pool that holds only a few molecules still completes every request, in place."""
    reqs = [W.water_cluster(m, seed=m) for m in range(20, 32)]
    srv = X.Server(pool_gib=0.03, max_slots=64, plain_workers=1, iters_per_step=4)
    ids = [srv.submit(Z, xyz) for Z, xyz in reqs]
    res = [srv.wait(i) for i in ids]
    st = srv.stats()
    srv.close()
    assert st["peak_resident"] < len(reqs)
    assert all(r.engine == 0 and r.status == 0 for r in res)
    p = plain(*reqs[-1])
    assert abs(res[-1].energy - p.energy) <= 1e-9
