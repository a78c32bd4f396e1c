"""Python host interface over the C ABI of libxtb_gb300.so.

Mirrors the reference C API (include/xtb.h) one call per method, so a caller
drives exactly the same sequence as a C program: environment -> molecule ->
calculator (GFN2-xTB) -> single point -> results getters.  Errors pushed onto
the environment are raised as ``XTBException`` after each call.

The library is loaded from this package directory; there is no fallback: if the
compiled engine is missing, importing the loader raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "libxtb_gb300.so")

_lib = None
PHASES = ("setup", "integrals", "cholesky", "hbuild", "stdform", "sytrd", "trieig", "backtransform", "density",
          "popmix", "gradient", "total")


class XTBException(RuntimeError):
    pass


def load_library(path=LIBPATH):
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise XTBException(f"{path} not found: build it with `python -m xtb_gb300.build`")
    lib = C.CDLL(path)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
    sig = {
        "xtb_getAPIVersion": (C.c_int, []),
        "xtb_newEnvironment": (vp, []),
        "xtb_delEnvironment": (None, [C.POINTER(vp)]),
        "xtb_checkEnvironment": (C.c_int, [vp]),
        "xtb_showEnvironment": (None, [vp, C.c_char_p]),
        "xtb_getError": (None, [vp, C.c_char_p, ip]),
        "xtb_setOutput": (None, [vp, C.c_char_p]),
        "xtb_releaseOutput": (None, [vp]),
        "xtb_setVerbosity": (None, [vp, C.c_int]),
        "xtb_newMolecule": (vp, [vp, ip, ip, dp, dp, ip, dp, C.POINTER(C.c_bool)]),
        "xtb_delMolecule": (None, [C.POINTER(vp)]),
        "xtb_updateMolecule": (None, [vp, vp, dp, dp]),
        "xtb_newCalculator": (vp, []),
        "xtb_delCalculator": (None, [C.POINTER(vp)]),
        "xtb_loadGFN2xTB": (None, [vp, vp, vp, C.c_char_p]),
        "xtb_setAccuracy": (None, [vp, vp, C.c_double]),
        "xtb_setMaxIter": (None, [vp, vp, C.c_int]),
        "xtb_setElectronicTemp": (None, [vp, vp, C.c_double]),
        "xtb_singlepoint": (None, [vp, vp, vp, vp]),
        "xtb_newResults": (vp, []),
        "xtb_delResults": (None, [C.POINTER(vp)]),
        "xtb_copyResults": (vp, [vp]),
        "xtb_getEnergy": (None, [vp, vp, dp]),
        "xtb_getGradient": (None, [vp, vp, dp]),
        "xtb_getCharges": (None, [vp, vp, dp]),
        "xtb_getDipole": (None, [vp, vp, dp]),
        "xtb_getBondOrders": (None, [vp, vp, dp]),
        "xtb_getNao": (None, [vp, vp, ip]),
        "xtb_getOrbitalEigenvalues": (None, [vp, vp, dp]),
        "xtb_getOrbitalOccupations": (None, [vp, vp, dp]),
        "xtb_getOrbitalCoefficients": (None, [vp, vp, dp]),
        "xtb_hessian": (None, [vp, vp, vp, vp, dp, ip, ip, dp, dp]),
        "xtb_getVirial": (None, [vp, vp, dp]),
        "xtb_getSolvationEnergy": (None, [vp, vp, dp]),
        "xtb_getPCGradient": (None, [vp, vp, dp]),
        "xtb_setExternalCharges": (None, [vp, vp, ip, ip, dp, dp]),
        "xtb_releaseExternalCharges": (None, [vp, vp]),
        "xtb_setSolvent": (None, [vp, vp, C.c_char_p, ip, dp, ip, C.c_char_p]),
        "xtb_releaseSolvent": (None, [vp, vp]),
        "xtbgb_getSolvationEnergyParts": (C.c_int, [vp, vp, dp]),
        "xtbgb_setSolventSalt": (None, [vp, vp, C.c_double, C.c_double]),
        "xtbgb_setSolventKernel": (None, [vp, vp, C.c_int]),
        "xtbgb_deviceCount": (C.c_int, []),
        "xtbgb_getIterations": (None, [vp, vp, ip, ip]),
        "xtbgb_getEnergyParts": (None, [vp, vp, dp]),
        "xtbgb_getShellCharges": (None, [vp, vp, dp]),
        "xtbgb_getMultipoles": (None, [vp, vp, dp, dp]),
        "xtbgb_getPhaseTimes": (None, [vp, vp, dp]),
        "xtbgb_getTransferBytes": (None, [vp, vp, C.POINTER(C.c_longlong)]),
        "xtbgb_setKeepOrbitals": (None, [vp, vp, C.c_int]),
        "xtbgb_setPrecision": (None, [vp, vp, C.c_int, C.c_int]),
        "xtbgb_setBlockedBacktransform": (None, [vp, vp, C.c_int]),
        "xtbgb_fp64PeakTflops": (C.c_double, []),
        "xtbgb_fp64PeakDetail": (None, [C.POINTER(C.c_double)]),
        "xtbgb_autotune": (C.c_int, [vp, dp, C.c_int]),
        "xtbgb_sytrdMs": (C.c_double, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
        "xtbgb_backtransformCheck": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, dp]),
        "xtbgb_setExternalChargesHardness": (None, [vp, vp, C.c_int, dp, dp, dp]),
        "xtbgb_writeRestart": (C.c_int, [vp, vp, vp, C.c_char_p]),
        "xtbgb_readRestart": (C.c_int, [vp, vp, vp, C.c_char_p]),
        "xtbgb_getTuning": (None, [vp, dp]),
        "xtbgb_setTuning": (None, [vp, C.c_int, C.c_int, C.c_int]),
        "xtbgb_fp64LatencyCycles": (None, [dp]),
        "xtbgb_reciprocalCheck": (C.c_int, [dp]),
        "xtbgb_splitGemmCheck": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, dp]),
        "xtbgb_repulsionNoAlloc": (C.c_int, [C.c_int, vp, vp, vp, vp, vp, C.c_char_p, C.c_int]),
        "xtbgb_newBatch": (vp, [vp, C.c_int, ip, ip, dp, dp, ip]),
        "xtbgb_delBatch": (None, [C.POINTER(vp)]),
        "xtbgb_batchSinglepoint": (None, [vp, vp, C.c_double, C.c_double, C.c_int, C.c_int]),
        "xtbgb_batchGetEnergies": (None, [vp, vp, dp]),
        "xtbgb_batchGetGradients": (None, [vp, vp, dp]),
        "xtbgb_batchGetCharges": (None, [vp, vp, dp]),
        "xtbgb_batchGetDipoles": (None, [vp, vp, dp]),
        "xtbgb_batchGetEnergyParts": (None, [vp, vp, dp]),
        "xtbgb_batchGetStatus": (None, [vp, vp, ip, ip, ip, ip]),
        "xtbgb_batchGetStats": (None, [vp, vp, dp, C.POINTER(C.c_longlong)]),
        "xtbgb_batchNao": (None, [vp, vp, ip]),
        "xtbgb_newServer": (vp, [vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]),
        "xtbgb_newServerEx": (vp, [vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                   C.c_int, C.c_int, C.c_int, C.c_int]),
        "xtbgb_delServer": (None, [C.POINTER(vp)]),
        "xtbgb_serverSubmit": (C.c_longlong, [vp, vp, C.c_int, ip, dp, C.c_double, C.c_int, C.c_int]),
        "xtbgb_serverWait": (C.c_int, [vp, vp, C.c_longlong, C.c_double, dp, dp, dp, dp]),
        "xtbgb_serverStats": (None, [vp, vp, dp]),
        "xtbgb_serverInjectAdmissionFailures": (None, [vp, vp, C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Environment:
    def __init__(self, verbosity=0):
        self.lib = load_library()
        self.h = C.c_void_p(self.lib.xtb_newEnvironment())
        self.lib.xtb_setVerbosity(self.h, verbosity)

    def check(self):
        if self.lib.xtb_checkEnvironment(self.h):
            buf = C.create_string_buffer(4096)
            n = C.c_int(4096)
            self.lib.xtb_getError(self.h, buf, C.byref(n))
            raise XTBException(buf.value.decode())

    def __del__(self):
        if getattr(self, "h", None) is not None and self.lib is not None:
            self.lib.xtb_delEnvironment(C.byref(self.h))


class Calculator:
    """GFN2-xTB single point through the C ABI (numbers, positions in Bohr)."""

    def __init__(self, numbers, positions, charge=0.0, uhf=0, accuracy=1.0, etemp=300.0, maxiter=250,
                 verbosity=0, keep_orbitals=True, precision="fp64", slices=5, blocked_min=None):
        self.lib = load_library()
        self.env = Environment(verbosity)
        self.numbers = np.ascontiguousarray(numbers, dtype=np.int32)
        self.positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        n = C.c_int(len(self.numbers))
        ch = C.c_double(charge)
        u = C.c_int(uhf)
        self.mol = C.c_void_p(self.lib.xtb_newMolecule(
            self.env.h, C.byref(n), self.numbers.ctypes.data_as(C.POINTER(C.c_int)), _dptr(self.positions),
            C.byref(ch), C.byref(u), None, None))
        self.env.check()
        self.calc = C.c_void_p(self.lib.xtb_newCalculator())
        self.lib.xtb_loadGFN2xTB(self.env.h, self.mol, self.calc, None)
        self.env.check()
        self.lib.xtb_setAccuracy(self.env.h, self.calc, accuracy)
        self.lib.xtb_setElectronicTemp(self.env.h, self.calc, etemp)
        self.lib.xtb_setMaxIter(self.env.h, self.calc, maxiter)
        self.lib.xtbgb_setKeepOrbitals(self.env.h, self.calc, int(bool(keep_orbitals)))
        self.lib.xtbgb_setPrecision(self.env.h, self.calc, 1 if precision == "split" else 0, slices)
        if blocked_min is not None:
            self.lib.xtbgb_setBlockedBacktransform(self.env.h, self.calc, int(blocked_min))
        self.env.check()
        self.res = C.c_void_p(self.lib.xtb_newResults())

    def set_external_charges(self, charges, positions, numbers=None, hardness=None):
        """External point charges (e, bohr): xtb_setExternalCharges with element numbers (the
        charges take those elements' hardness), or xtbgb_setExternalChargesHardness with explicit
        hardness values."""
        q = np.ascontiguousarray(charges, dtype=np.float64)
        x = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        n = len(q)
        if hardness is not None:
            g = np.ascontiguousarray(hardness, dtype=np.float64)
            self.lib.xtbgb_setExternalChargesHardness(self.env.h, self.calc, n, _dptr(q), _dptr(x), _dptr(g))
        else:
            z = np.ascontiguousarray(numbers, dtype=np.int32)
            nn = C.c_int(n)
            self.lib.xtb_setExternalCharges(self.env.h, self.calc, C.byref(nn), z.ctypes.data_as(C.POINTER(C.c_int)),
                                            _dptr(q), _dptr(x))
        self.env.check()
        self.npc = n

    def set_solvent(self, solvent, model="gbsa", state=None, temperature=None, grid=None, ion_strength=None,
                    ion_rad=None, kernel=None):
        """Implicit solvent (xtb_setSolvent): model "gbsa" or "alpb"; state 1 gsolv, 2 reference,
        3 1 bar; temperature in K; grid = Lebedev points per atom.  ion_strength (mol/L) and
        ion_rad (Bohr) switch on salt screening of the GBSA kernel (xtbgb_setSolventSalt);
        kernel "still" or "p16" replaces the model's Born kernel (xtbgb_setSolventKernel)."""
        if ion_strength is not None:
            self.lib.xtbgb_setSolventSalt(self.env.h, self.calc, float(ion_strength), float(ion_rad or 0.0))
            self.env.check()
        st = C.c_int(state) if state is not None else None
        tp = C.c_double(temperature) if temperature is not None else None
        gr = C.c_int(grid) if grid is not None else None
        self.lib.xtb_setSolvent(self.env.h, self.calc, solvent.encode(), C.byref(st) if st is not None else None,
                                C.byref(tp) if tp is not None else None, C.byref(gr) if gr is not None else None,
                                model.encode() if model is not None else None)
        self.env.check()
        if kernel is not None:
            self.lib.xtbgb_setSolventKernel(self.env.h, self.calc, {"still": 0, "p16": 1}[kernel])
            self.env.check()

    def release_solvent(self):
        self.lib.xtb_releaseSolvent(self.env.h, self.calc)
        self.env.check()

    def write_restart(self, path):
        """Write the last single point's wavefunction as an xtbrestart file (xtbgb_writeRestart)."""
        ok = self.lib.xtbgb_writeRestart(self.env.h, self.mol, self.res, str(path).encode())
        self.env.check()
        return bool(ok)

    def read_restart(self, path):
        """Load an xtbrestart file; the next singlepoint(fresh=False) starts from it. Returns
        whether the file matched the molecule (warnings stay on the environment)."""
        return bool(self.lib.xtbgb_readRestart(self.env.h, self.mol, self.res, str(path).encode()))

    def release_external_charges(self):
        self.lib.xtb_releaseExternalCharges(self.env.h, self.calc)
        self.env.check()
        self.npc = 0

    def update(self, positions):
        self.positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        self.lib.xtb_updateMolecule(self.env.h, self.mol, _dptr(self.positions), None)
        self.env.check()

    def shell_charges(self, nshell):
        out = np.zeros(nshell)
        self.lib.xtbgb_getShellCharges(self.env.h, self.res, _dptr(out))
        self.env.check()
        return out

    def hessian(self, fresh=True):
        """xtb_hessian: numerical Hessian [3N, 3N] (Eh/bohr^2) and dipole gradient [3N, 3];
        ``fresh`` starts from a new results object, as the reference's C test does."""
        if fresh:
            self.lib.xtb_delResults(C.byref(self.res))
            self.res = C.c_void_p(self.lib.xtb_newResults())
        n3 = 3 * len(self.numbers)
        hess = np.zeros((n3, n3))
        dipgrad = np.zeros((n3, 3))
        self.lib.xtb_hessian(self.env.h, self.mol, self.calc, self.res, _dptr(hess), None, None, _dptr(dipgrad), None)
        self.env.check()
        return hess, dipgrad

    def singlepoint(self, fresh=True):
        """Run xtb_singlepoint; ``fresh`` drops the warm-start wavefunction first."""
        if fresh:
            self.lib.xtb_delResults(C.byref(self.res))
            self.res = C.c_void_p(self.lib.xtb_newResults())
        self.lib.xtb_singlepoint(self.env.h, self.mol, self.calc, self.res)
        self.env.check()
        return Results(self)

    def __del__(self):
        lib = getattr(self, "lib", None)
        if lib is None:
            return
        for name, fn in (("res", lib.xtb_delResults), ("calc", lib.xtb_delCalculator), ("mol", lib.xtb_delMolecule)):
            h = getattr(self, name, None)
            if h is not None:
                fn(C.byref(h))


class Results:
    def __init__(self, calc):
        lib, env, res = calc.lib, calc.env, calc.res
        n = len(calc.numbers)
        e = C.c_double()
        lib.xtb_getEnergy(env.h, res, C.byref(e))
        self.energy = e.value
        self.gradient = np.zeros((n, 3))
        lib.xtb_getGradient(env.h, res, _dptr(self.gradient))
        self.charges = np.zeros(n)
        lib.xtb_getCharges(env.h, res, _dptr(self.charges))
        self.dipole = np.zeros(3)
        lib.xtb_getDipole(env.h, res, _dptr(self.dipole))
        nao = C.c_int()
        lib.xtb_getNao(env.h, res, C.byref(nao))
        self.nao = nao.value
        self.emo = np.zeros(self.nao)
        lib.xtb_getOrbitalEigenvalues(env.h, res, _dptr(self.emo))
        self.focc = np.zeros(self.nao)
        lib.xtb_getOrbitalOccupations(env.h, res, _dptr(self.focc))
        self.bond_orders = np.zeros((n, n))
        lib.xtb_getBondOrders(env.h, res, _dptr(self.bond_orders))
        it, conv = C.c_int(), C.c_int()
        lib.xtbgb_getIterations(env.h, res, C.byref(it), C.byref(conv))
        self.iterations, self.converged = it.value, bool(conv.value)
        parts = np.zeros(8)
        lib.xtbgb_getEnergyParts(env.h, res, _dptr(parts))
        (self.e_elec, self.e_rep, self.e_es, self.e_aes, self.e_axc, self.e_disp, self.e_atm,
         self.hl_gap) = parts
        self.gnorm = float(np.sqrt(np.sum(self.gradient ** 2)))
        self.phase_ms = np.zeros(len(PHASES))
        lib.xtbgb_getPhaseTimes(env.h, res, _dptr(self.phase_ms))
        sp = np.zeros(5)
        self.solvated = bool(lib.xtbgb_getSolvationEnergyParts(env.h, res, _dptr(sp)))
        self.g_solv, self.g_born, self.g_hb, self.g_sasa, self.g_shift = sp
        self.pcgrad = None
        if getattr(calc, "npc", 0):
            self.pcgrad = np.zeros((calc.npc, 3))
            lib.xtb_getPCGradient(env.h, res, _dptr(self.pcgrad))
        tb = (C.c_longlong * 3)()
        lib.xtbgb_getTransferBytes(env.h, res, tb)
        self.h2d_bytes, self.d2h_bytes, self.launches = int(tb[0]), int(tb[1]), int(tb[2])
        env.check()


class Batch:
    """Many GFN2-xTB single points in one call of the batched engine (xtbgb_newBatch ...).

    ``molecules`` is a list of (numbers, positions in Bohr); ``charges`` / ``uhf`` optional lists.
    """

    def __init__(self, molecules, charges=None, uhf=None, verbosity=0):
        self.lib = load_library()
        self.env = Environment(verbosity)
        self.natoms = np.array([len(z) for z, _ in molecules], dtype=np.int32)
        self.offsets = np.concatenate([[0], np.cumsum(self.natoms)])
        self.numbers = np.ascontiguousarray(np.concatenate([np.asarray(z, dtype=np.int32) for z, _ in molecules]))
        self.positions = np.ascontiguousarray(
            np.concatenate([np.asarray(x, dtype=np.float64).reshape(-1, 3) for _, x in molecules]))
        nmol = len(molecules)
        ch = None if charges is None else np.ascontiguousarray(charges, dtype=np.float64)
        uh = None if uhf is None else np.ascontiguousarray(uhf, dtype=np.int32)
        self.h = C.c_void_p(self.lib.xtbgb_newBatch(
            self.env.h, nmol, self.natoms.ctypes.data_as(C.POINTER(C.c_int)),
            self.numbers.ctypes.data_as(C.POINTER(C.c_int)), _dptr(self.positions),
            None if ch is None else _dptr(ch), None if uh is None else uh.ctypes.data_as(C.POINTER(C.c_int))))
        self.env.check()
        self.nmol = nmol
        self.nao = np.zeros(nmol, dtype=np.int32)
        self.lib.xtbgb_batchNao(self.env.h, self.h, self.nao.ctypes.data_as(C.POINTER(C.c_int)))

    def run(self, accuracy=1.0, etemp=300.0, maxiter=250, gradient=True, check=True):
        """Run every single point; returns a BatchResults.  With ``check`` an error on the
        environment (failed or unconverged molecules) raises after the results are read."""
        self.lib.xtbgb_batchSinglepoint(self.env.h, self.h, accuracy, etemp, maxiter, int(bool(gradient)))
        failed = self.lib.xtb_checkEnvironment(self.env.h)
        msg = None
        if failed:
            buf = C.create_string_buffer(4096)
            n = C.c_int(4096)
            self.lib.xtb_getError(self.env.h, buf, C.byref(n))
            msg = buf.value.decode()
            if "not available" in msg or "not allocated" in msg:
                raise XTBException(msg)
        r = BatchResults(self)
        r.error = msg
        if check and msg:
            raise XTBException(msg)
        return r

    def __del__(self):
        lib = getattr(self, "lib", None)
        if lib is not None and getattr(self, "h", None) is not None:
            lib.xtbgb_delBatch(C.byref(self.h))


class BatchResults:
    def __init__(self, b):
        lib, env, h, n = b.lib, b.env, b.h, b.nmol
        N = int(b.offsets[-1])
        ip = C.POINTER(C.c_int)
        self.energy = np.zeros(n)
        lib.xtbgb_batchGetEnergies(env.h, h, _dptr(self.energy))
        g = np.zeros((N, 3))
        lib.xtbgb_batchGetGradients(env.h, h, _dptr(g))
        q = np.zeros(N)
        lib.xtbgb_batchGetCharges(env.h, h, _dptr(q))
        self.gradients = [g[b.offsets[i]:b.offsets[i + 1]] for i in range(n)]
        self.charges = [q[b.offsets[i]:b.offsets[i + 1]] for i in range(n)]
        self.dipole = np.zeros((n, 3))
        lib.xtbgb_batchGetDipoles(env.h, h, _dptr(self.dipole))
        self.parts = np.zeros((n, 8))
        lib.xtbgb_batchGetEnergyParts(env.h, h, _dptr(self.parts))
        self.iterations = np.zeros(n, dtype=np.int32)
        self.converged = np.zeros(n, dtype=np.int32)
        self.status = np.zeros(n, dtype=np.int32)
        self.engine = np.zeros(n, dtype=np.int32)
        lib.xtbgb_batchGetStatus(env.h, h, self.iterations.ctypes.data_as(ip), self.converged.ctypes.data_as(ip),
                                 self.status.ctypes.data_as(ip), self.engine.ctypes.data_as(ip))
        t = np.zeros(2)
        c = (C.c_longlong * 4)()
        lib.xtbgb_batchGetStats(env.h, h, _dptr(t), c)
        self.device_ms, self.wall_ms = float(t[0]), float(t[1])
        self.h2d_bytes, self.d2h_bytes, self.launches, self.plain_count = (int(c[0]), int(c[1]), int(c[2]),
                                                                          int(c[3]))


class Server:
    """Request loop with continuous batching (xtbgb_newServer ...).

    ``submit`` returns a request id; ``wait`` returns a ServedResult.  Calls from several
    Python threads are safe: every call uses an environment of its own thread.  The defaults
    (six plain-engine workers, one SCC iteration per pool step) measured best on the mixed
    request stream of 3..1500 atoms.
    """

    def __init__(self, pool_gib=16.0, max_slots=1024, plain_workers=6, iters_per_step=1, accuracy=1.0,
                 etemp=300.0, maxiter=250, precision="fp64", slices=5, pool_max_nao=512, coop_blocks=0):
        import threading
        self.lib = load_library()
        self._tls = threading.local()
        env = self._env()
        self.h = C.c_void_p(self.lib.xtbgb_newServerEx(env.h, pool_gib, max_slots, plain_workers, iters_per_step,
                                                       accuracy, etemp, maxiter, 1 if precision == "split" else 0,
                                                       slices, int(pool_max_nao), int(coop_blocks)))
        env.check()
        self._natoms = {}

    def _env(self):
        e = getattr(self._tls, "env", None)
        if e is None:
            e = self._tls.env = Environment(0)
        return e

    def submit(self, numbers, positions, charge=0.0, uhf=0, gradient=True):
        env = self._env()
        z = np.ascontiguousarray(numbers, dtype=np.int32)
        x = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        rid = self.lib.xtbgb_serverSubmit(env.h, self.h, len(z), z.ctypes.data_as(C.POINTER(C.c_int)), _dptr(x),
                                          charge, uhf, int(bool(gradient)))
        env.check()
        self._natoms[rid] = len(z)
        return rid

    def wait(self, rid, timeout=-1.0, check=True):
        env = self._env()
        n = self._natoms[rid]
        e = C.c_double()
        g = np.zeros((n, 3))
        q = np.zeros(n)
        info = np.zeros(12)
        ok = self.lib.xtbgb_serverWait(env.h, self.h, rid, timeout, C.byref(e), _dptr(g), _dptr(q), _dptr(info))
        if not ok:
            return None
        err = None
        if self.lib.xtb_checkEnvironment(env.h):
            buf = C.create_string_buffer(4096)
            nb = C.c_int(4096)
            self.lib.xtb_getError(env.h, buf, C.byref(nb))
            err = buf.value.decode()
            if check:
                raise XTBException(err)
        del self._natoms[rid]
        return ServedResult(rid, e.value, g, q, info, err)

    def inject_admission_failures(self, count):
        """Test hook: the next `count` admissions to the resident pool fail on the host as if the
        device had run out of memory (xtbgb_serverInjectAdmissionFailures)."""
        env = self._env()
        self.lib.xtbgb_serverInjectAdmissionFailures(env.h, self.h, int(count))
        env.check()

    def stats(self):
        s = np.zeros(16)
        self.lib.xtbgb_serverStats(self._env().h, self.h, _dptr(s))
        keys = ("completed", "plain", "steps", "busy_s", "peak_resident", "reruns", "h2d_bytes", "d2h_bytes",
                "launches", "pool_scc_ms", "pool_scc_flops")
        return dict(zip(keys, s.tolist()))

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value is not None:
            self.lib.xtbgb_delServer(C.byref(self.h))

    def __del__(self):
        if getattr(self, "lib", None) is not None:
            self.close()


class ServedResult:
    def __init__(self, rid, energy, gradient, charges, info, error):
        self.id = rid
        self.energy = energy
        self.gradient = gradient
        self.charges = charges
        self.iterations, self.converged, self.status, self.engine = (int(v) for v in info[:4])
        self.t_submit, self.t_start, self.t_done = (float(v) for v in info[4:7])
        self.dipole = np.array(info[7:10])
        self.latency = self.t_done - self.t_submit
        self.nao = int(info[10])
        self.sytrd_ms = float(info[11])
        self.error = error


def autotune():
    """Measure the device's kernel-form crossovers (xtbgb_autotune) and return them with the
    timings behind them."""
    lib = load_library()
    env = Environment(0)
    out = np.zeros(256)
    m = lib.xtbgb_autotune(env.h, _dptr(out), len(out))
    env.check()
    v = out[:m]
    r1 = int(v[4])
    rows1 = v[5:5 + 3 * r1].reshape(r1, 3)
    r2 = int(v[5 + 3 * r1])
    rows2 = v[6 + 3 * r1:6 + 3 * r1 + 4 * r2].reshape(r2, 4)
    return {"sytrd_sym_min": int(v[0]), "blocked_min_fp64": int(v[1]), "blocked_min_split": int(v[2]),
            "seconds": float(v[3]),
            "sytrd_ms": [{"n": int(a), "row_form": b, "upper_triangle_form": c} for a, b, c in rows1],
            "backtransform_ms": [{"n": int(a), "warp_form": b, "blocked_fp64": c, "blocked_split": d}
                                 for a, b, c, d in rows2]}


def sytrd_ms(n, form=-1, max_blocks=0, reps=3):
    """CUDA-event time (ms, best of reps) of one tridiagonalisation of a random symmetric n x n
    matrix (xtbgb_sytrdMs): form 0 row form, 1 upper-triangle form, -1 the tuned choice;
    max_blocks > 0 caps the cooperative grid."""
    lib = load_library()
    env = Environment(0)
    ms = lib.xtbgb_sytrdMs(env.h, int(n), int(form), int(max_blocks), int(reps))
    env.check()
    return float(ms)


def backtransform_check(n, ncol, slices=0):
    """Compact-WY eigenvector back-transformation (slices 0: FP64 column strips, > 0: split
    products) against the one-warp-per-vector form on ncol columns of a random n x n matrix
    (xtbgb_backtransformCheck): (max |difference| / max |Z|, warp-form ms, compact-WY ms)."""
    lib = load_library()
    env = Environment(0)
    out = np.zeros(3)
    rc = lib.xtbgb_backtransformCheck(env.h, int(n), int(ncol), int(slices), _dptr(out))
    env.check()
    if rc != 0:
        raise XTBException("xtbgb_backtransformCheck failed")
    return float(out[0]), float(out[1]), float(out[2])


def get_tuning():
    lib = load_library()
    env = Environment(0)
    out = np.zeros(4)
    lib.xtbgb_getTuning(env.h, _dptr(out))
    return {"sytrd_sym_min": int(out[0]), "blocked_min_fp64": int(out[1]), "blocked_min_split": int(out[2]),
            "measured": bool(out[3])}


def set_tuning(sytrd_sym_min, blocked_min_fp64, blocked_min_split):
    lib = load_library()
    env = Environment(0)
    lib.xtbgb_setTuning(env.h, int(sytrd_sym_min), int(blocked_min_fp64), int(blocked_min_split))
    env.check()
