"""GFN2-xTB parameter set for the CPU oracle (test infrastructure only).

Loads ``xtb_gb300/data/gfn2_params.json`` (generated from the reference by
``oracle/gen_params.py``) and derives the per-shell tables the reference builds
at start-up:

* ``initHamiltonian``      src/xtb/gfn2.f90:809-866   (kScale, enScale, valence shells)
* ``setGFN2ReferenceOcc``  src/xtb/gfn2.f90:869-890
* ``setGFN2NumberOfPrimitives`` src/xtb/gfn2.f90:893-937
* ``setGFN2ThirdOrderShell``    src/xtb/gfn2.f90:940-967
* ``setGFN1ShellHardness``      src/xtb/gfn1.f90:845-871
* ``angToShellData`` / ``generateValenceShellData`` src/xtb/data.f90:469-703
"""
import json
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_JSON = os.path.join(os.path.dirname(_HERE), "xtb_gb300", "data", "gfn2_params.json")

# physical constants, src/mctc/convert.f90:25-29 and src/mctc/mctc_constants.f90:22-34
AUTOAA = 0.52917726
AATOAU = 1.0 / AUTOAA
AUTOEV = 27.21138505
EVTOAU = 1.0 / AUTOEV
KB = 3.166808578545117e-06
PI = 3.1415926535897932384626433832795029

# GFN2 global parameters, src/xtb/gfn2.f90:44-66
KSHELL = np.array([1.85, 2.23, 2.23, 2.23])
ENSHELL = 2.0
KSD = 2.0
KPD = 2.0
GAM3SHELL = np.array([[1.0, 0.5, 0.25, 0.25], [1.0, 0.5, 0.25, 0.25]])  # (kind, l)
AES_SHIFT, AES_EXP, AES_RMAX = 1.2, 4.0, 5.0
AES_DMP3, AES_DMP5 = 3.0, 4.0
GEXP = 2.0                              # alphaj: Klopman-Ohno exponent
D4_S6, D4_S8, D4_S10, D4_A1, D4_A2, D4_S9, D4_ALP = 1.0, 2.7, 0.0, 0.52, 5.0, 5.0, 16
D4_GA, D4_GC, D4_WF = 3.0, 2.0, 6.0     # src/xtb/gfn2.f90:762-774
REP_KEXP, REP_KEXP_LIGHT, REP_REXP = 1.5, 1.0, 1.0


class Params:
    def __init__(self, path=_JSON):
        raw = json.load(open(path))
        for k, v in raw.items():
            if isinstance(v, dict):
                a = np.array(v["data"], dtype=np.float64 if v["dtype"].startswith("float") else np.int64)
                setattr(self, k, a.reshape(v["shape"]))
            else:
                setattr(self, k, v)
        self._derive()

    def _derive(self):
        nel = self.maxElem
        self.kScale = np.zeros((4, 4))
        for i in range(4):
            for j in range(4):
                self.kScale[j, i] = 0.5 * (KSHELL[i] + KSHELL[j])
        self.kScale[0, 2] = self.kScale[2, 0] = KSD
        self.kScale[1, 2] = self.kScale[2, 1] = KPD
        self.enScale = np.full((4, 4), 0.005 * (ENSHELL + ENSHELL))
        # per-shell tables (shell index, element index 0-based)
        self.valenceShell = np.zeros((3, nel), dtype=np.int64)
        self.referenceOcc = np.zeros((3, nel))
        self.numberOfPrimitives = np.zeros((3, nel), dtype=np.int64)
        self.kCN = np.zeros((3, nel))
        self.shellPoly = np.zeros((3, nel))
        self.thirdOrderShell = np.zeros((3, nel))
        self.shellHardnessSh = np.zeros((3, nel))
        for iz in range(nel):
            seen = set()
            for ish in range(self.nShell[iz]):
                l = self.angShell[ish, iz]
                if l not in seen:
                    seen.add(l)
                    self.valenceShell[ish, iz] = 1
                if self.valenceShell[ish, iz]:
                    self.referenceOcc[ish, iz] = self.referenceOccL[l, iz]
                n = self.principalQuantumNumber[ish, iz]
                if iz + 1 <= 2:
                    nprim = {0: 3, 1: 4}.get(l, 0)
                else:
                    nprim = {0: 6 if n > 5 else 4, 1: 6 if n > 5 else 4, 2: 3, 3: 4}[l]
                self.numberOfPrimitives[ish, iz] = nprim
                self.kCN[ish, iz] = self.kCNL[l, iz]
                self.shellPoly[ish, iz] = self.shellPolyL[l, iz]
                kind = self.gfn2Kinds[iz]
                self.thirdOrderShell[ish, iz] = self.thirdOrderAtom[iz] * GAM3SHELL[kind - 1, l]
                self.shellHardnessSh[ish, iz] = self.chemicalHardness[iz] * (1.0 + self.shellHardness[l, iz])


def valence_charge(Z):
    """Valence (core-less) nuclear charge, src/type/molecule.f90:559-596."""
    z = np.asarray(Z)
    core = np.select([z <= 2, z <= 10, z <= 18, z <= 29, z <= 36, z <= 47, z <= 54, z <= 71, z <= 79, z <= 86],
                     [0, 2, 10, 18, 28, 36, 46, 54, 68, 78], 86)
    val = (z - core).astype(np.float64)
    val[(z > 57) & (z < 72)] = 3.0
    return val


_PARAMS = None


def get_params():
    global _PARAMS
    if _PARAMS is None:
        _PARAMS = Params()
    return _PARAMS
