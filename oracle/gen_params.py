"""Extract the GFN2-xTB parameter tables from the reference's Fortran sources.

Test infrastructure.  This script reads the reference tree (default
``/root/reference``) and writes two committed artefacts:

* ``xtb_gb300/data/gfn2_params.json`` -- every per-element table the GFN2
  single point needs (Hamiltonian, Coulomb, multipole, repulsion, D4, EEQ,
  STO-nG expansion), already scaled to the units the reference uses at run
  time;
* ``xtb_gb300/csrc/gfn2_params.inc`` -- the same numbers as C arrays for the
  device engine.

The numbers are the published GFN2-xTB / D4 / EEQ-2019 / Stewart STO-nG
parameter sets; they have to be bit-identical to the reference's for parity,
so they are parsed, not retyped.  Fortran default-real literals (no ``_wp``
kind suffix) are single precision in the reference and are rounded through
float32 here, exactly as the Fortran compiler does.

Sources (paths relative to the reference root):
  src/xtb/gfn2.f90                      GFN2 per-element data (:98-725)
  src/xtb/data.f90                      valenceCN, multiRad (:330-366)
  src/param/{atomicrad,paulingen,covalentradd3,sqrtzr4r2}.f90
  src/disp/ncoord.f90                   single-precision covalent radii / EN (:66-111)
  src/charge_model.f90                  EEQ 2019 model (:147-245)
  src/mctc/param/chemical_hardnesses.f90  D4 chemical hardness
  src/disp/dftd4_parameters.f90         D4 effective charges (:36-47)
  include/param_ref.fh                  D4 reference polarisabilities
  src/slater.f90                        Stewart 1970 STO-nG tables (:33-367)
"""
import json
import os
import re
import sys

import numpy as np

REF = os.environ.get("XTB_REFERENCE", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)

NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eEdD][-+]?\d+)?(?:_[wW][pP])?")


def _strip_comments(text):
    out = []
    for line in text.splitlines():
        i = line.find("!")
        if i >= 0:
            line = line[:i]
        out.append(line)
    return "\n".join(out)


def _to_float(tok):
    dbl = tok.lower().endswith("_wp")
    core = tok[:-3] if dbl else tok
    core = core.replace("d", "e").replace("D", "e")
    v = float(core)
    if not dbl and ("." in core or "e" in core.lower()):
        v = float(np.float32(v))          # default REAL literal: single precision
    return v


def _numbers(body):
    return [_to_float(t) for t in NUM.findall(body)]


def fortran_array(path, name):
    """Return (values, trailing_expression) of ``name(...) = <array literal> [expr]``."""
    src = _strip_comments(open(os.path.join(REF, path)).read())
    m = re.search(r"::\s*" + re.escape(name) + r"\s*\([^)]*\)\s*=", src)
    if m is None:
        raise KeyError(f"{name} not found in {path}")
    i = m.end()
    # the statement continues while lines end with '&'
    stmt = []
    for line in src[i:].splitlines():
        s = line.rstrip()
        if not s.strip() and stmt:
            continue                      # comment-only continuation line
        stmt.append(s)
        if not s.endswith("&"):
            break
    text = " ".join(x.rstrip("&").lstrip().lstrip("&") for x in stmt)
    # array body between the first [ or (/ and its matching close
    ia, ib = text.find("["), text.find("(/")
    if ia >= 0 and (ib < 0 or ia < ib):
        a = ia
        b = text.index("]", a)
    else:
        a = ib + 1
        b = text.index("/)", a)
    body = text[a + 1:b]
    rest = text[b + 1:]
    return _numbers(body), rest, text[:a]


def col_major(vals, shape):
    return np.array(vals, dtype=np.float64).reshape(shape[::-1]).T


def scaled(path, name, factor_ops=()):
    """Array values with the trailing scale factors written in the source applied.

    ``factor_ops`` lists the (op, value) pairs the source statement is expected
    to carry after the array literal; a mismatch with the source raises.
    """
    vals, rest, _ = fortran_array(path, name)
    x = np.array(vals, dtype=np.float64)
    rest = re.sub(r",\s*shape\(\s*\w+\s*\)\s*\)", "", rest).strip().strip(")").strip()
    found = [(op, _to_float(num)) for op, num in re.findall(r"([*/])\s*([-+0-9.eEdD_wWpP]+)", rest)]
    if [(op, v) for op, v in found] != [(op, float(c)) for op, c in factor_ops]:
        raise ValueError(f"{name}: source scale {rest!r} != expected {factor_ops}")
    for op, c in factor_ops:
        x = x * c if op == "*" else x / c
    return x


AUTOAA = 0.52917726
AATOAU = 1.0 / AUTOAA


def parse_param_ref():
    """Parse the ``data`` statements of include/param_ref.fh."""
    src = _strip_comments(open(os.path.join(REF, "include/param_ref.fh")).read())
    src = src.replace("&\n", " ").replace("\n     &", " ")
    stmts = re.findall(r"data\s+(\w+)\s*\(([^)]*)\)\s*/([^/]*)/", src)
    refn = np.zeros(118, dtype=np.int64)
    arr7 = {k: np.zeros((7, 118)) for k in ("refq", "refh", "hcount", "ascale", "refcovcn", "refcn")}
    refsys = np.zeros((7, 118), dtype=np.int64)
    alphaiw = np.zeros((23, 7, 118))
    sscale = np.zeros(17)
    secaiw = np.zeros((23, 17))
    for name, idx, body in stmts:
        name = name.lower()
        idx = [s.strip() for s in idx.split(",")]
        vals = _numbers(body)
        if name == "refn":
            refn[int(idx[0]) - 1] = int(vals[0])
        elif name in arr7:
            arr7[name][int(idx[0]) - 1, int(idx[1]) - 1] = vals[0]
        elif name == "refsys":
            refsys[int(idx[0]) - 1, int(idx[1]) - 1] = int(vals[0])
        elif name == "alphaiw":
            assert idx[0] == ":" and len(vals) == 23
            alphaiw[:, int(idx[1]) - 1, int(idx[2]) - 1] = vals
        elif name == "sscale":
            sscale[int(idx[0]) - 1] = vals[0]
        elif name == "secaiw":
            assert idx[0] == ":" and len(vals) == 23
            secaiw[:, int(idx[1]) - 1] = vals
    return refn, arr7, refsys, alphaiw, sscale, secaiw


def main():
    g2 = "src/xtb/gfn2.f90"
    P = {}
    maxel = 86
    P["maxElem"] = maxel
    P["repAlpha"] = scaled(g2, "repAlpha")
    P["repZeff"] = scaled(g2, "repZeff")
    P["chemicalHardness"] = scaled(g2, "chemicalHardness")
    P["thirdOrderAtom"] = scaled(g2, "thirdOrderAtom", [("*", 0.1)])
    P["shellHardness"] = col_major(scaled(g2, "shellHardness"), (3, maxel))
    P["dipKernel"] = scaled(g2, "dipKernel", [("*", 0.01)])
    P["quadKernel"] = scaled(g2, "quadKernel", [("*", 0.01)])
    P["nShell"] = scaled(g2, "nShell").astype(np.int64)
    P["angShell"] = col_major(scaled(g2, "angShell"), (3, maxel)).astype(np.int64)
    P["principalQuantumNumber"] = col_major(scaled(g2, "principalQuantumNumber"), (3, maxel)).astype(np.int64)
    P["referenceOccL"] = col_major(scaled(g2, "referenceOcc"), (3, maxel))
    P["shellPolyL"] = col_major(scaled(g2, "shellPoly"), (4, maxel))
    P["kCNL"] = col_major(scaled(g2, "kCN"), (4, maxel))
    P["selfEnergy"] = col_major(scaled(g2, "selfEnergy"), (3, maxel))
    P["slaterExponent"] = col_major(scaled(g2, "slaterExponent"), (3, maxel))
    P["gfn2Kinds"] = scaled(g2, "gfn2Kinds").astype(np.int64)

    P["valenceCN"] = scaled("src/xtb/data.f90", "valenceCN")
    P["multiRad"] = scaled("src/xtb/data.f90", "multiRad")
    # atomicRad = aatoau * [..]
    P["atomicRad"] = AATOAU * scaled("src/param/atomicrad.f90", "atomicRad")
    P["paulingEN"] = scaled("src/param/paulingen.f90", "paulingEN")
    # covalentRadD3 = [..] * aatoau * 4.0_wp / 3.0_wp
    x, rest, _ = fortran_array("src/param/covalentradd3.f90", "covalentRadD3")
    assert rest.replace(" ", "") == "*aatoau*4.0_wp/3.0_wp", rest
    P["covalentRadD3"] = ((np.array(x) * AATOAU) * 4.0) / 3.0
    r4 = scaled("src/param/sqrtzr4r2.f90", "r4Overr2")
    z = np.arange(1, 119, dtype=np.float64)
    P["sqrtZr4r2"] = np.sqrt(0.5 * (r4 * np.sqrt(z)))
    # ncoord.f90: single precision radii and EN; rcov = 4.0_wp/3.0_wp*rad/0.52917726_wp
    rad = scaled("src/disp/ncoord.f90", "rad")
    P["rcovD4"] = ((4.0 / 3.0) * rad) / 0.52917726
    P["enD4"] = scaled("src/disp/ncoord.f90", "en")
    # EEQ 2019 (first model in charge_model.f90)
    src = open(os.path.join(REF, "src/charge_model.f90")).read()
    start = src.index("subroutine new_charge_model_2019")
    stop = src.index("end subroutine new_charge_model_2019")
    block = _strip_comments(src[start:stop])
    for key in ("en", "gam", "kappa", "alpha"):
        m = re.search(r"::\s*" + key + r"\s*\(max_elem\)\s*=\s*\(/(.*?)/\)", block, re.S)
        P["eeq_" + key] = np.array(_numbers(m.group(1).replace("&", " ")))
    P["d4_gam"] = scaled("src/mctc/param/chemical_hardnesses.f90", "chemical_hardness")
    P["d4_zeff"] = scaled("src/disp/dftd4_parameters.f90", "zeff")
    refn, arr7, refsys, alphaiw, sscale, secaiw = parse_param_ref()
    P["d4_refn"] = refn
    for k, v in arr7.items():
        P["d4_" + k] = v
    P["d4_refsys"] = refsys
    P["d4_alphaiw"] = alphaiw
    P["d4_sscale"] = sscale
    P["d4_secaiw"] = secaiw
    # Stewart STO-nG
    sl = "src/slater.f90"
    P["sto_alpha1"] = scaled(sl, "pAlpha1")
    for ng in range(2, 7):
        P[f"sto_alpha{ng}"] = col_major(scaled(sl, f"pAlpha{ng}"), (ng, 15))
        P[f"sto_coeff{ng}"] = col_major(scaled(sl, f"pCoeff{ng}"), (ng, 15))
    for k in ("pAlpha6s", "pCoeff6s", "pAlpha6p", "pCoeff6p"):
        P["sto_" + k] = scaled(sl, k)

    out = {}
    for k, v in P.items():
        if isinstance(v, np.ndarray):
            out[k] = {"shape": list(v.shape), "dtype": str(v.dtype),
                      "data": [float(t) if v.dtype.kind == "f" else int(t) for t in v.ravel(order="C")]}
        else:
            out[k] = v
    dst = os.path.join(REPO, "xtb_gb300", "data", "gfn2_params.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=0)
    write_c_tables(P, os.path.join(REPO, "xtb_gb300", "csrc", "gfn2_params.inc"))
    print("wrote", dst)


def write_c_tables(P, dst):
    """Emit the per-element tables the device engine reads (row-major C layout)."""
    lines = ["// Generated by oracle/gen_params.py from the reference parameter sources.",
             "// GFN2-xTB (Bannwarth, Ehlert, Grimme 2019), D4, EEQ-2019 and Stewart STO-nG data.",
             "#pragma once", ""]

    def emit(name, arr, ctype="double"):
        a = np.asarray(arr)
        flat = a.ravel(order="C")
        dims = "".join(f"[{d}]" for d in a.shape)
        if ctype == "double":
            body = ", ".join(repr(float(x)) for x in flat)
        else:
            body = ", ".join(str(int(x)) for x in flat)
        lines.append(f"static const {ctype} k_{name}{dims} = {{{body}}};")

    for k, v in P.items():
        if not isinstance(v, np.ndarray):
            continue
        emit(k, v, "double" if v.dtype.kind == "f" else "int")
    with open(dst, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    sys.exit(main())
