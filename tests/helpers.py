"""Shared helpers: golden fixtures and tolerances."""
import json
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "gfn2_reference.json")
AUTOEV = 27.21138505

# parity tolerances of the GFN2 single point (energy Eh, charges e, gradient Eh/bohr, SCC iterations)
TOL_E = 1e-6
TOL_Q = 1e-5
TOL_G = 1e-5
TOL_ITER = 1


def golden():
    return json.load(open(GOLDEN))


def case_geometry(case):
    return np.array(case["numbers"]), np.array(case["positions"], dtype=float).reshape(-1, 3)


def evaluate(expr, r):
    """Value of a reference test expression for a result object with energy, gradient, q, ... fields."""
    simple = {"res%e_total": "energy", "energy": "energy", "res%gnorm": "gnorm", "norm2(gradient)": "gnorm",
              "res%hl_gap": "hl_gap", "hl_gap": "hl_gap", "res%e_elec": "e_elec", "res%e_es": "e_es",
              "res%e_aes": "e_aes", "res%e_axc": "e_axc", "res%e_disp": "e_disp", "res%e_rep": "e_rep"}
    if expr in simple:
        return getattr(r, simple[expr])
    m = re.fullmatch(r"gradient\((\d),(\d+)\)", expr)
    if m:
        return r.gradient[int(m.group(2)) - 1, int(m.group(1)) - 1]
    m = re.fullmatch(r"wfn%(q|qsh)\((\d+)\)", expr)
    if m:
        return getattr(r, m.group(1))[int(m.group(2)) - 1]
    m = re.fullmatch(r"wfn%(dipm|qp)\((\d),(\d+)\)", expr)
    if m:
        return getattr(r, m.group(1))[int(m.group(3)) - 1, int(m.group(2)) - 1]
    if expr == "wfn%emo(wfn%ihomo)":
        return r.emo[r.ihomo - 1]
    if expr == "wfn%focc(wfn%ihomo)":
        return r.focc[r.ihomo - 1]
    if expr == "norm2(calc%pcem%grd)":
        return float(np.linalg.norm(r.pcgrad))
    m = re.fullmatch(r"calc%pcem%grd\((\d),(\d+)\)", expr)
    if m:
        return r.pcgrad[int(m.group(2)) - 1, int(m.group(1)) - 1]
    m = re.fullmatch(r"(grad|pcgrad)\[(\d+)\]", expr)
    if m:
        return (r.gradient if m.group(1) == "grad" else r.pcgrad).ravel()[int(m.group(2))]
    m = re.fullmatch(r"(q|dipole)\[(\d+)\]", expr)
    if m:
        name = m.group(1)
        vals = getattr(r, name) if hasattr(r, name) else r.charges     # engine results name them charges
        return vals[int(m.group(2))]
    m = re.fullmatch(r"wbo\[(\d+)\]", expr)
    if m:
        wbo = r.wbo if hasattr(r, "wbo") else r.bond_orders
        return wbo.ravel()[int(m.group(1))]
    raise KeyError(expr)
