"""Batched engine (one thread block per molecule) against the plain engine and the oracle.

Tolerances: the parity bar against the oracle (|dE| <= 1e-6 Eh, charges <= 1e-5 e,
gradient <= 1e-5 Eh/bohr, SCC iterations +-1).  Against the plain GPU engine, which runs
the same device arithmetic in a different launch shape (only summation orders differ),
the bar is tighter: |dE| <= 1e-9 Eh, charges and gradient <= 1e-7.
"""
import numpy as np
import pytest

from helpers import TOL_E, TOL_G, TOL_ITER, TOL_Q
from oracle import gfn2
from xtb_gb300 import interface as X
from xtb_gb300 import workloads as W

TIGHT_E, TIGHT_QG = 1e-9, 1e-7

SMALL = {
    "hydroxide": ([8, 1], [[0.0, 0.0, 0.0], [0.0, 0.0, 1.83]], -1, 0),
    "ammonium": ([7, 1, 1, 1, 1], [[0, 0, 0], [1.12, 1.12, 1.12], [-1.12, -1.12, 1.12], [-1.12, 1.12, -1.12],
                                   [1.12, -1.12, -1.12]], 1, 0),
    "methyl_radical": ([6, 1, 1, 1], [[0, 0, 0], [2.04, 0, 0], [-1.02, 1.767, 0], [-1.02, -1.767, 0.05]], 0, 1),
    "h2": ([1, 1], [[0, 0, 0], [0, 0, 1.4]], 0, 0),
}


def mixed_set():
    mols, ch, uh, names = [], [], [], []
    for n in (1, 3, 7, 12):
        mols.append(W.alkane(n, 0.02, seed=10 + n))
        ch.append(0.0), uh.append(0), names.append(f"C{n}")
    for m in (2, 5, 9, 16):
        mols.append(W.water_cluster(m, seed=20 + m))
        ch.append(0.0), uh.append(0), names.append(f"W{m}")
    for k, (z, x, c, u) in SMALL.items():
        mols.append((np.array(z), np.array(x, dtype=float)))
        ch.append(float(c)), uh.append(u), names.append(k)
    return mols, ch, uh, names


def plain(Z, xyz, charge=0.0, uhf=0):
    return X.Calculator(Z, xyz, charge=charge, uhf=uhf, keep_orbitals=False).singlepoint()


@pytest.fixture(scope="module")
def mixed():
    mols, ch, uh, names = mixed_set()
    r = X.Batch(mols, charges=ch, uhf=uh).run()
    return mols, ch, uh, names, r


@pytest.mark.gpu
def test_batch_matches_plain_engine(mixed):
    mols, ch, uh, names, r = mixed
    assert np.all(r.status == 0) and np.all(r.converged == 1)
    assert np.all(r.engine == 0)
    for i, ((Z, xyz), c, u) in enumerate(zip(mols, ch, uh)):
        p = plain(Z, xyz, c, u)
        assert abs(r.energy[i] - p.energy) <= TIGHT_E, (names[i], r.energy[i], p.energy)
        assert np.max(np.abs(r.charges[i] - p.charges)) <= TIGHT_QG, names[i]
        assert np.max(np.abs(r.gradients[i] - p.gradient)) <= TIGHT_QG, names[i]
        assert abs(int(r.iterations[i]) - p.iterations) <= TOL_ITER, names[i]
        assert np.max(np.abs(r.dipole[i] - p.dipole)) <= 1e-7, names[i]
        parts = np.array([p.e_elec, p.e_rep, p.e_es, p.e_aes, p.e_axc, p.e_disp, p.e_atm])
        assert np.max(np.abs(r.parts[i, :7] - parts)) <= TIGHT_E, names[i]


@pytest.mark.gpu
@pytest.mark.parametrize("idx", [2, 6, 9])
def test_batch_matches_oracle(mixed, idx):
    mols, ch, uh, names, r = mixed
    Z, xyz = mols[idx]
    o = gfn2.singlepoint(np.asarray(Z), np.asarray(xyz, dtype=float), charge=ch[idx], uhf=uh[idx])
    assert abs(r.energy[idx] - o.energy) <= TOL_E
    assert np.max(np.abs(r.charges[idx] - o.q)) <= TOL_Q
    assert np.max(np.abs(r.gradients[idx] - o.gradient)) <= TOL_G
    assert abs(int(r.iterations[idx]) - o.iterations) <= TOL_ITER


@pytest.mark.gpu
def test_alone_equals_in_the_mix(mixed):
    """A molecule's result does not depend on the other molecules of its batch."""
    mols, ch, uh, names, r = mixed
    for i in (0, 5, 10):
        alone = X.Batch([mols[i]], charges=[ch[i]], uhf=[uh[i]]).run()
        assert abs(alone.energy[0] - r.energy[i]) <= 1e-12, names[i]
        assert np.max(np.abs(alone.charges[0] - r.charges[i])) <= 1e-12
        assert np.max(np.abs(alone.gradients[0] - r.gradients[i])) <= 1e-10   # atomic gradient sums
        assert alone.iterations[0] == r.iterations[i]


@pytest.mark.gpu
def test_energy_only_and_repeat(mixed):
    mols, ch, uh, names, r = mixed
    b = X.Batch(mols, charges=ch, uhf=uh)
    e1 = b.run(gradient=False)
    e2 = b.run(gradient=True)
    assert np.max(np.abs(e1.energy - r.energy)) <= 1e-12
    assert np.max(np.abs(e2.energy - r.energy)) <= 1e-12
    assert e2.launches > 0 and e2.device_ms > 0.0


@pytest.mark.gpu
def test_hot_smearing_matches_plain_engine():
    """At 20000 K the occupations reach past the levels the batched SCC bisects first (nocc +
    max(8, n / 8)): the block bisects the rest and smears again, and the batch still matches
    the plain engine."""
    mols = [W.water_cluster(m, seed=20 + m) for m in (3, 8)] + [W.alkane(6, 0.02, seed=4)]
    r = X.Batch(mols).run(etemp=20000.0)
    assert np.all(r.status == 0) and np.all(r.engine == 0)
    for i, (Z, xyz) in enumerate(mols):
        p = X.Calculator(Z, xyz, etemp=20000.0).singlepoint()
        assert abs(r.energy[i] - p.energy) <= TIGHT_E
        assert np.max(np.abs(r.charges[i] - p.charges)) <= TIGHT_QG
        assert np.max(np.abs(r.gradients[i] - p.gradient)) <= TIGHT_QG


@pytest.mark.gpu
def test_large_molecule_runs_on_plain_engine():
    big = W.water_cluster(90, seed=3)                 # 540 AOs, above the batched limit
    small = W.alkane(4, 0.02, seed=4)
    r = X.Batch([small, big]).run()
    assert list(r.engine) == [0, 1] and r.plain_count == 1
    p = plain(*big)
    assert abs(r.energy[1] - p.energy) <= 1e-12
    assert np.max(np.abs(r.gradients[1] - p.gradient)) <= 1e-12


def test_batch_rejects_bad_input():
    """Argument checks run on the host (no device call)."""
    with pytest.raises(X.XTBException, match="not parametrised"):
        X.Batch([(np.array([87, 1]), np.zeros((2, 3)))])
    with pytest.raises(X.XTBException, match="no atoms"):
        X.Batch([(np.array([], dtype=np.int32), np.zeros((0, 3)))])
