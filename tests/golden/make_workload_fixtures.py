"""Oracle results for the seeded benchmark geometries, stored as golden fixtures.

The workloads have no reference-side values (they are generated here), so the
oracle -- itself pinned to the reference's known-answer tests -- provides the
expected energy, charges, gradient and SCC iteration count.

Usage: python tests/golden/make_workload_fixtures.py [name ...]
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import gfn2  # noqa: E402
from xtb_gb300 import workloads as W  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

FIXTURES = {
    "c10h22_seed1": lambda: W.alkane(10, 0.02, seed=1),
    "h2o_30_seed1": lambda: W.water_cluster(30, seed=1),
    "c50h102_seed3": lambda: W.alkane(50, 0.02, seed=3),
    "h2o_300_seed1": lambda: W.water_cluster(300, seed=1),
    "c200h402_seed1": lambda: W.alkane(200, 0.02, seed=1),
}


def make(name):
    Z, xyz = FIXTURES[name]()
    t = time.time()
    r = gfn2.singlepoint(Z, xyz)
    dt = time.time() - t
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), numbers=Z, positions=xyz, energy=r.energy,
                        charges=r.q, gradient=r.gradient, iterations=r.iterations, dipole=r.dipole,
                        emo=r.emo, oracle_seconds=dt)
    print(f"{name}: E = {r.energy:.10f}  iterations = {r.iterations}  ({dt:.1f} s)")


if __name__ == "__main__":
    for n in (sys.argv[1:] or list(FIXTURES)):
        make(n)
