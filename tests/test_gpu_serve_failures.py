"""Failure handling of the request loop, with every failure made on the host.

The reference's convention (src/type/environment.f90:162-195, src/scf_module.F90:806-808) is
that a failing single point reports an error and never aborts the caller.  The request loop
must keep that per request: a request that cannot be admitted, a request that is invalid and
a molecule whose SCC does not converge each complete with an error status, and the requests
around them are served as usual.  Nothing here faults the GPU: admission failures come from a
host-side hook, invalid molecules are refused before any device work, and the unconverged
case is a small maxiter.
"""
import numpy as np
import pytest

from xtb_gb300 import interface as X
from xtb_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def small_molecules():
    return [W.water_cluster(3, seed=1), W.alkane(4, 0.02, seed=2), W.water_cluster(5, seed=3),
            W.alkane(6, 0.02, seed=4), W.water_cluster(4, seed=5), W.alkane(3, 0.02, seed=6)]


def test_admission_failure_fails_only_that_request():
    mols = small_molecules()
    srv = X.Server(pool_gib=1.0, max_slots=16, plain_workers=1, iters_per_step=2)
    srv.inject_admission_failures(2)
    ids = [srv.submit(Z, xyz) for Z, xyz in mols]
    res = [srv.wait(i, check=False) for i in ids]
    failed = [r for r in res if r.status != 0]
    assert len(failed) == 2
    for r in failed:
        assert r.status == 3 and "admission failed" in r.error
    # admission runs in arrival order: the first two requests took the injected failures
    assert [r.status for r in res[:2]] == [3, 3]
    for (Z, xyz), r in zip(mols[2:], res[2:]):
        p = X.Calculator(Z, xyz, keep_orbitals=False).singlepoint()
        assert r.error is None and r.converged == 1
        assert abs(r.energy - p.energy) <= 1e-9
    # the pool's budget came back: a second round admits everything
    again = [srv.wait(srv.submit(Z, xyz)) for Z, xyz in mols]
    assert all(r.status == 0 for r in again)
    srv.close()


@pytest.mark.parametrize("case", ["z0", "unparametrised", "coincident", "nonfinite"])
def test_invalid_request_is_refused_and_the_server_goes_on(case):
    Z, xyz = W.water_cluster(3, seed=7)
    Z, xyz = np.array(Z), np.array(xyz)
    if case == "z0":
        Z[1] = 0
        msg = "not parametrised"
    elif case == "unparametrised":
        Z[0] = 87
        msg = "not parametrised"
    elif case == "coincident":
        xyz[4] = xyz[1]
        msg = "coincide"
    else:
        xyz[2, 1] = np.nan
        msg = "non-finite"
    srv = X.Server(pool_gib=1.0, max_slots=8, plain_workers=1)
    with pytest.raises(X.XTBException, match=msg):
        srv.submit(Z, xyz)
    good = srv.wait(srv.submit(*W.water_cluster(3, seed=7)))
    assert good.status == 0 and good.converged == 1
    srv.close()


def test_invalid_molecule_refused_by_the_drop_in_call():
    """xtb_singlepoint pushes the same error on the environment (no device work is done)."""
    Z, xyz = W.alkane(3, 0.02, seed=1)
    xyz = np.array(xyz)
    xyz[5] = xyz[0]
    with pytest.raises(X.XTBException, match="coincide"):
        X.Calculator(Z, xyz).singlepoint()


def test_unconverged_requests_report_an_error():
    """maxiter = 2: a pool molecule and a plain-engine molecule both end unconverged, with the
    reference's error text, finite energies, and the server still serving."""
    srv = X.Server(pool_gib=1.0, max_slots=8, plain_workers=1, maxiter=2)
    small = W.water_cluster(6, seed=2)           # 36 AOs: resident pool
    large = W.water_cluster(90, seed=3)          # 540 AOs: plain-engine worker
    rs = srv.wait(srv.submit(*small), check=False)
    rl = srv.wait(srv.submit(*large), check=False)
    for r, engine in ((rs, 0), (rl, 1)):
        assert r.engine == engine
        assert r.status == 1 and r.converged == 0
        assert "did not converge" in r.error
        assert np.isfinite(r.energy) and r.iterations == 2
    srv.close()
