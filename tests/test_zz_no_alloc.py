"""Allocation-free repulsion entry point (xtbgb_repulsionNoAlloc).

The entry point takes device pointers and works in a static device scratch array.
Its energy is compared with the repulsion energy the engine reports through the
C ABI (xtb_singlepoint + xtbgb_getEnergyParts) on two calls in a row -- a larger
molecule, then a smaller one, so stale scratch from the first call would show --
and its gradient with central differences of its own energy.  The file is named
to be collected last, so it also runs after every other test in the same process.
"""
import ctypes as C

import numpy as np
import pytest

from xtb_gb300 import interface as X
from xtb_gb300 import workloads as W

MAX_ATOMS = 8192


def _device_buffers(torch, Z, xyz):
    dev = torch.device("cuda:0")
    z = torch.as_tensor(np.asarray(Z, dtype=np.int32), device=dev)
    x = torch.as_tensor(np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1), device=dev)
    e = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    g = torch.full((len(Z), 3), float("nan"), dtype=torch.float64, device=dev)
    return z, x, e, g


def _call(lib, torch, bufs):
    z, x, e, g = bufs
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(torch.device("cuda:0")).cuda_stream
    rc = lib.xtbgb_repulsionNoAlloc(z.numel(), z.data_ptr(), x.data_ptr(), e.data_ptr(), g.data_ptr(),
                                    stream or None, err, len(err))
    assert rc == 0, err.value.decode()


def _engine_erep(Z, xyz):
    calc = X.Calculator(Z, xyz, keep_orbitals=False)
    return calc.singlepoint().e_rep


def test_rejects_sizes_beyond_scratch():
    """Size checks come before any device call, so this runs without a GPU."""
    lib = X.load_library()
    err = C.create_string_buffer(256)
    for n in (0, -3, MAX_ATOMS + 1):
        rc = lib.xtbgb_repulsionNoAlloc(n, None, None, None, None, None, err, len(err))
        assert rc != 0
        assert b"8192" in err.value
    rc = lib.xtbgb_repulsionNoAlloc(4, None, None, None, None, None, err, len(err))
    assert rc != 0 and b"null" in err.value


@pytest.mark.gpu
def test_two_calls_match_engine_repulsion_and_allocate_nothing():
    torch = pytest.importorskip("torch")
    lib = X.load_library()
    cases = [W.water_cluster(30, seed=1), W.alkane(10, 0.02, seed=1)]   # larger first, then smaller
    ref = [_engine_erep(Z, xyz) for Z, xyz in cases]
    bufs = [_device_buffers(torch, Z, xyz) for Z, xyz in cases]
    _call(lib, torch, bufs[1])                 # set-up call (symbol lookup) before measuring
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for b in bufs:                             # two calls in a row
        _call(lib, torch, b)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    for (z, x, e, g), er, (Z, _) in zip(bufs, ref, cases):
        ev = float(e.item())
        assert abs(ev - er) <= 1e-12 * max(1.0, abs(er)), (ev, er)
        gv = g.cpu().numpy()
        assert np.all(np.isfinite(gv)) and gv.shape == (len(Z), 3)
        assert abs(gv.sum(axis=0)).max() < 1e-10       # pair forces cancel


@pytest.mark.gpu
def test_repeat_is_bitwise_and_gradient_matches_finite_differences():
    torch = pytest.importorskip("torch")
    lib = X.load_library()
    Z, xyz = W.alkane(10, 0.02, seed=1)
    bufs = _device_buffers(torch, Z, xyz)
    _call(lib, torch, bufs)
    e1, g1 = float(bufs[2].item()), bufs[3].cpu().numpy()
    _call(lib, torch, bufs)
    e2, g2 = float(bufs[2].item()), bufs[3].cpu().numpy()
    assert e1 == e2 and np.array_equal(g1, g2)
    h = 1e-4
    for atom, k in ((0, 0), (5, 1), (17, 2), (31, 0)):
        es = []
        for sgn in (1.0, -1.0):
            p = np.array(xyz, dtype=np.float64).copy()
            p[atom, k] += sgn * h
            b = _device_buffers(torch, Z, p)
            _call(lib, torch, b)
            es.append(float(b[2].item()))
        fd = (es[0] - es[1]) / (2 * h)
        assert abs(fd - g1[atom, k]) < 1e-7, (atom, k, fd, g1[atom, k])
