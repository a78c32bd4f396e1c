"""The C ABI library: load, exported symbols, handle life cycle and error
convention of the reference API (runs on CPU, no device calls)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from xtb_gb300 import interface as X

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in ("xtb.h", "xtb_gb300.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(xtb(?:gb)?_[A-Za-z]+)\s*\(", src))
    names.discard("xtb_delete")
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    return X.load_library()


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 38
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_api_version(lib):
    assert lib.xtb_getAPIVersion() == 20000


def test_null_environment_is_a_noop(lib):
    n = C.c_int(1)
    z = np.array([1], dtype=np.int32)
    xyz = np.zeros(3)
    mol = lib.xtb_newMolecule(None, C.byref(n), z.ctypes.data_as(C.POINTER(C.c_int)),
                              xyz.ctypes.data_as(C.POINTER(C.c_double)), None, None, None, None)
    assert mol is None
    assert lib.xtb_checkEnvironment(None) == 0


def test_handles_are_nulled_on_delete(lib):
    env = C.c_void_p(lib.xtb_newEnvironment())
    calc = C.c_void_p(lib.xtb_newCalculator())
    res = C.c_void_p(lib.xtb_newResults())
    lib.xtb_delCalculator(C.byref(calc))
    lib.xtb_delResults(C.byref(res))
    lib.xtb_delEnvironment(C.byref(env))
    assert calc.value is None and res.value is None and env.value is None


def _error_text(lib, env):
    buf = C.create_string_buffer(1024)
    n = C.c_int(1024)
    lib.xtb_getError(env, buf, C.byref(n))
    return buf.value.decode()


def test_invalid_molecules_push_errors(lib):
    env = C.c_void_p(lib.xtb_newEnvironment())
    z = np.array([1, 0], dtype=np.int32)
    xyz = np.zeros(6)
    n = C.c_int(0)
    assert lib.xtb_newMolecule(env, C.byref(n), z.ctypes.data_as(C.POINTER(C.c_int)),
                               xyz.ctypes.data_as(C.POINTER(C.c_double)), None, None, None, None) is None
    assert lib.xtb_checkEnvironment(env) == 1
    assert "Number of atoms must be positive" in _error_text(lib, env)
    assert lib.xtb_checkEnvironment(env) == 0          # getError empties the log
    n = C.c_int(2)
    assert lib.xtb_newMolecule(env, C.byref(n), z.ctypes.data_as(C.POINTER(C.c_int)),
                               xyz.ctypes.data_as(C.POINTER(C.c_double)), None, None, None, None) is None
    assert "Invalid atomic number" in _error_text(lib, env)
    lib.xtb_delEnvironment(C.byref(env))


def test_call_order_errors(lib):
    env = C.c_void_p(lib.xtb_newEnvironment())
    z = np.array([8, 1, 1], dtype=np.int32)
    xyz = np.array([0.0, 0.0, -0.7, 1.4, 0.0, 0.4, -1.4, 0.0, 0.4])
    n = C.c_int(3)
    mol = C.c_void_p(lib.xtb_newMolecule(env, C.byref(n), z.ctypes.data_as(C.POINTER(C.c_int)),
                                         xyz.ctypes.data_as(C.POINTER(C.c_double)), None, None, None, None))
    calc = C.c_void_p(lib.xtb_newCalculator())
    res = C.c_void_p(lib.xtb_newResults())
    e = C.c_double()
    lib.xtb_getEnergy(env, res, C.byref(e))             # before any single point
    assert lib.xtb_checkEnvironment(env) == 1
    _error_text(lib, env)
    lib.xtb_singlepoint(env, mol, calc, res)            # no parametrisation loaded
    assert "No calculator loaded" in _error_text(lib, env)
    lib.xtb_setAccuracy(env, calc, 1.0)
    assert "no calculator loaded" in _error_text(lib, env)
    lib.xtb_loadGFN2xTB(env, mol, calc, None)
    assert lib.xtb_checkEnvironment(env) == 0
    lib.xtb_setAccuracy(env, calc, 1e6)                 # clamped with a warning, not an error
    assert lib.xtb_checkEnvironment(env) == 0
    lib.xtb_loadGFN1xTB(env, mol, calc, None)
    assert "not supported" in _error_text(lib, env)
    lib.xtb_singlepoint(env, mol, calc, None)
    assert "Calculation results are not allocated" in _error_text(lib, env)
    for h, f in ((res, lib.xtb_delResults), (calc, lib.xtb_delCalculator), (mol, lib.xtb_delMolecule)):
        f(C.byref(h))
    lib.xtb_delEnvironment(C.byref(env))


def test_unparametrised_element_is_rejected(lib):
    env = C.c_void_p(lib.xtb_newEnvironment())
    z = np.array([87], dtype=np.int32)
    xyz = np.zeros(3)
    n = C.c_int(1)
    mol = C.c_void_p(lib.xtb_newMolecule(env, C.byref(n), z.ctypes.data_as(C.POINTER(C.c_int)),
                                         xyz.ctypes.data_as(C.POINTER(C.c_double)), None, None, None, None))
    calc = C.c_void_p(lib.xtb_newCalculator())
    lib.xtb_loadGFN2xTB(env, mol, calc, None)
    assert "not parametrised" in _error_text(lib, env)
    lib.xtb_delCalculator(C.byref(calc))
    lib.xtb_delMolecule(C.byref(mol))
    lib.xtb_delEnvironment(C.byref(env))
