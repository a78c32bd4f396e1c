"""External point charges through the drop-in (needs a GB300).

The values the reference asserts for a water dimer in the field of six charges
(test/unit/test_gfn2.f90:459-520 with GFN2 hardnesses and with gamma = 999, and
test/api/c_api_example.c:298-410 through xtb_setExternalCharges) at the reference's own
thresholds, and agreement with the oracle on a larger cluster in a field of 30 charges.
"""
import numpy as np
import pytest

from helpers import TOL_E, TOL_G, TOL_Q, case_geometry, evaluate, golden
from oracle import gfn2
from oracle.params import get_params
from xtb_gb300 import interface as X
from xtb_gb300 import workloads as W

pytestmark = pytest.mark.gpu
CASES = golden()


@pytest.mark.parametrize("key", ["pcem_charges", "pcem_point", "capi_pc"])
def test_reference_point_charge_values(key):
    case = CASES[key]
    Z, xyz = case_geometry(case)
    calc = X.Calculator(Z, xyz, maxiter=case["maxiter"])
    if "pc_numbers" in case:
        calc.set_external_charges(case["pc_charges"], case["pc_positions"], numbers=case["pc_numbers"])
    else:
        calc.set_external_charges(case["pc_charges"], case["pc_positions"], hardness=case["pc_gam"])
    r = calc.singlepoint()
    assert r.converged
    for c in case["checks"]:
        got = evaluate(c["expr"], r)
        assert abs(got - c["value"]) <= max(c["thr"], 2e-10), (c["expr"], got, c["value"])


def test_point_charges_match_oracle_and_release():
    Z, xyz = W.water_cluster(12, seed=4)
    rng = np.random.default_rng(3)
    pcx = xyz.mean(axis=0) + rng.normal(0.0, 9.0, size=(30, 3))
    pcq = rng.uniform(-0.8, 0.8, 30)
    numbers = rng.choice([1, 6, 8], 30)
    gam = [get_params().chemicalHardness[z - 1] for z in numbers]
    calc = X.Calculator(Z, xyz)
    calc.set_external_charges(pcq, pcx, numbers=numbers)
    r = calc.singlepoint()
    o = gfn2.singlepoint(Z, xyz, pc_charges=pcq, pc_positions=pcx, pc_gam=gam)
    assert abs(r.energy - o.energy) <= TOL_E
    assert np.max(np.abs(r.charges - o.q)) <= TOL_Q
    assert np.max(np.abs(r.gradient - o.gradient)) <= TOL_G
    assert np.max(np.abs(r.pcgrad - o.pcgrad)) <= TOL_G
    # released: the plain single point again
    calc.release_external_charges()
    r0 = calc.singlepoint()
    o0 = gfn2.singlepoint(Z, xyz)
    assert abs(r0.energy - o0.energy) <= TOL_E


def test_invalid_external_charges_are_refused():
    Z, xyz = W.water_cluster(2, seed=1)
    calc = X.Calculator(Z, xyz)
    with pytest.raises(X.XTBException, match="Invalid element"):
        calc.set_external_charges([0.1], [[9.0, 0.0, 0.0]], numbers=[0])
    with pytest.raises(X.XTBException, match="invalid charge, position or hardness"):
        calc.set_external_charges([0.1], [[np.nan, 0.0, 0.0]], hardness=[0.4])
