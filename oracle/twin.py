"""C++/OpenMP + LAPACK twin of the CPU oracle (test and baseline infrastructure only).

``oracle/twin.cpp`` restates ``oracle.gfn2.singlepoint`` (the reference's ``scf``,
src/scf_module.F90:74-920, and ``scc``, src/scc_core.f90:255-640) with OpenMP loops and the
reference's LAPACK sequence (``dpotrf`` once; ``dsygst`` + ``dsyevd`` + ``dtrsm`` per SCC
iteration, src/mctc/lapack/eigensolve.F90:218-246; the density as one full ``dgemm``,
src/scc_core.f90:1177-1205).  It exists so that the reference's CPU algorithm can be timed on
every molecule of a workload, up to a few thousand orbitals, where the NumPy oracle takes
minutes.  This module gathers the per-atom and per-shell parameters (from ``oracle.params``,
the same tables the NumPy oracle uses), hands the C++ code the Fortran-ABI LAPACK/BLAS entry
points that SciPy exports, and returns a result with the oracle's field names.

The library is built by ``make -C oracle`` (``__graft_entry__.build()`` runs it).
"""
import ctypes as C
import os
import subprocess

import numpy as np

from . import gfn2
from . import integrals as I
from .params import get_params, valence_charge

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libgfn2twin.so")
MAXREF = 7

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class TwinInput(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("nat", "nsh", "nao", "maxprim", "nelem", "maxiter", "ihomoa", "ihomob")] + \
               [(k, C.c_double) for k in ("charge", "etemp", "accuracy")] + \
               [("xyz", _dp), ("Z", _ip)] + \
               [(k, _dp) for k in ("zval", "en", "covd3", "rcovd4", "end4", "eeq_en", "eeq_gam", "eeq_kappa",
                                   "eeq_alpha", "multirad", "valcn", "dipk", "quadk", "sqrtzr4r2", "atomicrad",
                                   "rep_alpha", "rep_zeff")] + \
               [(k, _ip) for k in ("d4_nref", "d4_off", "eidx")] + \
               [(k, _dp) for k in ("d4_zeff", "d4_gam", "d4_refcn", "d4_refq")] + \
               [("d4_ncount", _ip), ("c6ref", _dp)] + \
               [(k, _ip) for k in ("sh_atom", "sh_l", "sh_nprim", "sh_ao")] + \
               [(k, _dp) for k in ("alpha", "coef", "zeta", "se0", "kcn", "shpoly", "gam3", "eta", "zsh",
                                   "kscale", "enscale")] + \
               [("guess_eeq", C.c_int)]


class TwinLapack(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("dpotrf", "dsygst", "dsyevd", "dsysv", "dtrsm", "dgemm")]


class TwinOutput(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("energy", "e_elec", "e_rep", "e_es", "e_aes", "e_axc", "e_disp")] + \
               [("iterations", C.c_int), ("converged", C.c_int)] + \
               [(k, _dp) for k in ("q", "qsh", "gradient", "dipole", "wbo", "emo", "focc")] + \
               [("seconds", C.c_double * 4)]


_lib = None
_lapack = None


def build():
    """Compile libgfn2twin.so in place (g++ -O3 -fopenmp; no BLAS linked)."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the C++ twin failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def _capsule_pointer(cap):
    C.pythonapi.PyCapsule_GetName.restype = C.c_char_p
    C.pythonapi.PyCapsule_GetName.argtypes = [C.py_object]
    C.pythonapi.PyCapsule_GetPointer.restype = C.c_void_p
    C.pythonapi.PyCapsule_GetPointer.argtypes = [C.py_object, C.c_char_p]
    return C.pythonapi.PyCapsule_GetPointer(cap, C.pythonapi.PyCapsule_GetName(cap))


def lapack_pointers():
    """Fortran-ABI LAPACK/BLAS entry points exported by SciPy (its bundled OpenBLAS)."""
    global _lapack
    if _lapack is None:
        import scipy.linalg.cython_blas as B
        import scipy.linalg.cython_lapack as L
        t = TwinLapack()
        for name in ("dpotrf", "dsygst", "dsyevd", "dsysv"):
            setattr(t, name, _capsule_pointer(L.__pyx_capi__[name]))
        for name in ("dtrsm", "dgemm"):
            setattr(t, name, _capsule_pointer(B.__pyx_capi__[name]))
        _lapack = t
    return _lapack


def load():
    global _lib
    if _lib is None:
        # sleeping (not spinning) OpenMP workers leave the cores to OpenBLAS's own threads
        # between parallel regions; libgomp reads this when it is first loaded
        os.environ.setdefault("OMP_WAIT_POLICY", "passive")
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        lib.twin_singlepoint.argtypes = [C.POINTER(TwinInput), C.POINTER(TwinLapack), C.POINTER(TwinOutput)]
        lib.twin_singlepoint.restype = C.c_int
        _lib = lib
    return _lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Result:
    pass


def singlepoint(Z, xyz, charge=0.0, uhf=0, etemp=300.0, accuracy=1.0, maxiter=250, guess="eeq", wbo=False):
    """GFN2-xTB energy, charges, gradient (Bohr in; Eh, e, Eh/bohr out), as oracle.gfn2.singlepoint
    (guess "eeq" or "zero"); the returned object carries the same field names."""
    lib = load()
    Pr = get_params()
    Z = np.asarray(Z, dtype=np.int64)
    xyz = _d(np.asarray(xyz, dtype=np.float64).reshape(-1, 3))
    n = len(Z)
    iz = Z - 1
    basis = I.Basis(Z)
    zval = valence_charge(Z)
    nel = int(round(np.sum(zval) - charge))
    nopen = uhf
    if nopen == 0 and nel % 2 != 0:
        nopen = 1
    _, _, ihomoa, ihomob = gfn2.occu(basis.nao, nel, nopen)
    # D4 reference data per atom (newD4Model, src/disp/dftd4.F90:106-203)
    model = gfn2.D4Model(Z)
    elems = model.elements
    eidx = np.array([elems.index(int(z)) for z in Z])
    ne = len(elems)
    c6ref = np.zeros((ne, ne, MAXREF, MAXREF))
    for a, za in enumerate(elems):
        for b, zb in enumerate(elems):
            m = model.c6[za, zb]
            c6ref[a, b, :m.shape[0], :m.shape[1]] = m
    nref = np.array([model.nref[int(z)] for z in Z])
    off = np.concatenate([[0], np.cumsum(nref)[:-1]])
    refcn = np.concatenate([model.refcn[int(z)] for z in Z])
    refq = np.concatenate([model.q[int(z)] for z in Z])
    ncount = np.concatenate([model.ncount[int(z)] for z in Z])
    sh_z = iz[basis.sh_atom]
    keep = dict(
        xyz=xyz, Z=_i(Z), zval=_d(zval), en=_d(Pr.paulingEN[iz]), covd3=_d(Pr.covalentRadD3[iz]),
        rcovd4=_d(Pr.rcovD4[iz]), end4=_d(Pr.enD4[iz]), eeq_en=_d(Pr.eeq_en[iz]), eeq_gam=_d(Pr.eeq_gam[iz]),
        eeq_kappa=_d(Pr.eeq_kappa[iz]), eeq_alpha=_d(Pr.eeq_alpha[iz]), multirad=_d(Pr.multiRad[iz]),
        valcn=_d(Pr.valenceCN[iz]), dipk=_d(Pr.dipKernel[iz]), quadk=_d(Pr.quadKernel[iz]),
        sqrtzr4r2=_d(Pr.sqrtZr4r2[iz]), atomicrad=_d(Pr.atomicRad[iz]), rep_alpha=_d(Pr.repAlpha[iz]),
        rep_zeff=_d(Pr.repZeff[iz]), d4_nref=_i(nref), d4_off=_i(off), eidx=_i(eidx),
        d4_zeff=_d(Pr.d4_zeff[iz]), d4_gam=_d(Pr.d4_gam[iz]), d4_refcn=_d(refcn), d4_refq=_d(refq),
        d4_ncount=_i(ncount), c6ref=_d(c6ref),
        sh_atom=_i(basis.sh_atom), sh_l=_i(basis.sh_l), sh_nprim=_i(basis.sh_nprim), sh_ao=_i(basis.sh_ao),
        alpha=_d(basis.alpha), coef=_d(basis.coef), zeta=_d(basis.sh_zeta),
        se0=_d(Pr.selfEnergy[basis.sh_ish, sh_z]), kcn=_d(Pr.kCN[basis.sh_ish, sh_z]),
        shpoly=_d(Pr.shellPoly[basis.sh_ish, sh_z]), gam3=_d(Pr.thirdOrderShell[basis.sh_ish, sh_z]),
        eta=_d(Pr.shellHardnessSh[basis.sh_ish, sh_z]), zsh=_d(gfn2.set_zshell(basis, zval)),
        kscale=_d(Pr.kScale), enscale=_d(Pr.enScale))
    t = TwinInput(nat=n, nsh=basis.nshell, nao=basis.nao, maxprim=basis.alpha.shape[1], nelem=ne,
                  maxiter=maxiter, ihomoa=ihomoa, ihomob=ihomob, charge=charge, etemp=etemp, accuracy=accuracy,
                  guess_eeq=1 if guess == "eeq" else 0)
    for k, v in keep.items():
        setattr(t, k, v.ctypes.data_as(_ip if v.dtype == np.int32 else _dp))
    r = Result()
    r.q = np.zeros(n)
    r.qsh = np.zeros(basis.nshell)
    r.gradient = np.zeros((n, 3))
    r.dipole = np.zeros(3)
    r.wbo = np.zeros((n, n)) if wbo else None
    r.emo = np.zeros(basis.nao)
    r.focc = np.zeros(basis.nao)
    o = TwinOutput(q=r.q.ctypes.data_as(_dp), qsh=r.qsh.ctypes.data_as(_dp), gradient=r.gradient.ctypes.data_as(_dp),
                   dipole=r.dipole.ctypes.data_as(_dp), wbo=r.wbo.ctypes.data_as(_dp) if wbo else None,
                   emo=r.emo.ctypes.data_as(_dp), focc=r.focc.ctypes.data_as(_dp))
    rc = lib.twin_singlepoint(C.byref(t), C.byref(lapack_pointers()), C.byref(o))
    if rc == 1:
        raise RuntimeError("EEQ: Coulomb matrix is singular")
    if rc != 0:
        raise RuntimeError("Diagonalization of Hamiltonian failed")
    for k in ("energy", "e_elec", "e_rep", "e_es", "e_aes", "e_axc", "e_disp"):
        setattr(r, k, getattr(o, k))
    r.iterations = o.iterations
    r.converged = bool(o.converged)
    r.seconds = list(o.seconds)
    r.gnorm = float(np.sqrt(np.sum(r.gradient ** 2)))
    r.ihomo = ihomoa
    r.hl_gap = r.emo[ihomoa] - r.emo[ihomoa - 1] if 0 < ihomoa < basis.nao else 0.0
    r.nao = basis.nao
    r.nshell = basis.nshell
    return r
