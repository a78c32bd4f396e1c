"""xtbrestart files (src/restart.f90:33-86, 182-200).

The file is Fortran unformatted sequential: every record framed by its 4-byte length.  Record 1
holds six 64-bit integers (method twice, atoms, shells, electrons, unpaired electrons), record 2
the shell charges, records 3 and 4 (GFN2) the atomic dipoles (3, atoms) and quadrupoles
(6, atoms).  The round trip through the library runs on the host; the warm start from a written
file needs a GPU.
"""
import struct

import numpy as np
import pytest

from xtb_gb300 import interface as X
from xtb_gb300 import workloads as W


def record(payload):
    return struct.pack("<i", len(payload)) + payload + struct.pack("<i", len(payload))


def restart_bytes(nat, nsh, nel, nopen, qsh, dipm, qp, version=2):
    head = struct.pack("<6q", version, version, nat, nsh, nel, nopen)
    return (record(head) + record(np.asarray(qsh, dtype="<f8").tobytes()) +
            record(np.asarray(dipm, dtype="<f8").tobytes()) + record(np.asarray(qp, dtype="<f8").tobytes()))


def water_dimer():
    Z, xyz = W.water_cluster(2, seed=3)
    return np.asarray(Z), np.asarray(xyz)


@pytest.fixture()
def lib_or_skip():
    try:
        return X.load_library()
    except X.XTBException as e:
        pytest.skip(str(e))


def test_restart_round_trip_on_the_host(tmp_path, lib_or_skip):
    Z, xyz = water_dimer()                      # 2 x (O: 2 shells, H: 1 shell) = 8 shells, 16 electrons
    rng = np.random.default_rng(1)
    qsh, dipm, qp = rng.normal(size=8), rng.normal(size=(6, 3)), rng.normal(size=(6, 6))
    src = tmp_path / "xtbrestart"
    src.write_bytes(restart_bytes(6, 8, 16, 0, qsh, dipm, qp))
    calc = X.Calculator(Z, xyz)
    assert calc.read_restart(src)
    out = tmp_path / "xtbrestart.out"
    assert calc.write_restart(out)
    assert out.read_bytes() == src.read_bytes()


def test_restart_dimension_mismatch_is_not_loaded(tmp_path, lib_or_skip):
    Z, xyz = water_dimer()
    bad = tmp_path / "xtbrestart"
    bad.write_bytes(restart_bytes(7, 9, 18, 0, np.zeros(9), np.zeros((7, 3)), np.zeros((7, 6))))
    calc = X.Calculator(Z, xyz)
    assert not calc.read_restart(bad)
    assert not calc.read_restart(tmp_path / "missing")


@pytest.mark.gpu
def test_restart_warm_start(tmp_path):
    Z, xyz = W.water_cluster(20, seed=6)
    a = X.Calculator(Z, xyz)
    ra = a.singlepoint()
    path = tmp_path / "xtbrestart"
    assert a.write_restart(path)
    data = path.read_bytes()
    head = struct.unpack("<6q", data[4:52])
    assert head[:4] == (2, 2, len(Z), 80) and head[5] == 0     # 20 x (O: 2 shells, 2 H: 1 shell each)
    b = X.Calculator(Z, xyz)
    assert b.read_restart(path)
    rb = b.singlepoint(fresh=False)               # starts from the file's charges and moments
    assert abs(rb.energy - ra.energy) <= 1e-8
    assert rb.iterations < ra.iterations
