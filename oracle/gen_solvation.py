"""Extract the GBSA / ALPB implicit-solvation tables from the reference's sources.

Test infrastructure, like ``gen_params.py`` beside it: it reads the reference tree (default
``/root/reference``) and writes two committed artefacts,

* ``xtb_gb300/data/solvation_params.json`` -- for the oracle;
* ``xtb_gb300/csrc/solvation_params.inc`` -- the same numbers as C tables for the host side of
  the engine.

What is extracted (paths relative to the reference root):
  include/param_gbsa_<solvent>.fh   GFN2 GBSA parameter sets ``gfn2_<solvent>``
  include/param_alpb_<solvent>.fh   GFN2 ALPB parameter sets ``gfn2_alpb_<solvent>``
      each set: epsv, smass, rhos, c1, rprobe, gshift, soset, alpha, then per element (94)
      gamscale, sx and tmp (src/solv/model.f90:94-106)
  src/param/vdwradd3.f90            D3 van der Waals radii (``aatoau * [...]``, :37)
  src/solv/lebedev.f90              the Lebedev-Laikov angular grids: per grid the list of
      octahedral orbit generators (kind 1..6 with their a, b and weight v), :35-38, :319-...

The numbers are published parameter sets and quadrature tables; they must be the reference's
bit for bit, so they are parsed, not retyped.  The orbit expansion of a generator (the points
of an Oh orbit) is written independently in the oracle and in the engine.
"""
import json
import os
import re

import numpy as np

REF = os.environ.get("XTB_REFERENCE", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)

NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eEdD][-+]?\d+)?_wp")
AUTOAA = 0.52917726
AATOAU = 1.0 / AUTOAA
SCALARS = ["epsv", "smass", "rhos", "c1", "rprobe", "gshift", "soset", "alpha"]


def _strip(text):
    return "\n".join(line.split("!", 1)[0] for line in text.splitlines())


def _num(tok):
    return float(tok[:-3].replace("d", "e").replace("D", "e"))


def parameter_sets(prefix, model):
    """{solvent: parameters} of every ``gfn2_[alpb_]<solvent>`` set in include/param_<model>_*.fh."""
    out = {}
    inc = os.path.join(REF, "include")
    for fn in sorted(os.listdir(inc)):
        if not (fn.startswith(f"param_{model}_") and fn.endswith(".fh")):
            continue
        src = _strip(open(os.path.join(inc, fn)).read())
        for m in re.finditer(r"::\s*(\w+)\s*=\s*gbsa_parameter\s*\(", src):
            name = m.group(1)
            if not name.startswith(prefix):
                continue
            end = src.find("type(gbsa_parameter)", m.end())
            vals = [_num(t) for t in NUM.findall(src[m.end():end if end > 0 else len(src)])]
            if len(vals) != len(SCALARS) + 3 * 94:
                raise ValueError(f"{fn}:{name}: {len(vals)} numbers")
            p = dict(zip(SCALARS, vals[:len(SCALARS)]))
            k = len(SCALARS)
            p["gamscale"], p["sx"], p["tmp"] = vals[k:k + 94], vals[k + 94:k + 188], vals[k + 188:]
            out[name[len(prefix):]] = p
    return out


def vdw_rad_d3():
    src = _strip(open(os.path.join(REF, "src/param/vdwradd3.f90")).read())
    m = re.search(r"vanDerWaalsRadD3\(1:94\)\s*=\s*aatoau\s*\*\s*\[", src)
    body = src[m.end():src.index("]", m.end())]
    vals = [_num(t) for t in NUM.findall(body)]
    assert len(vals) == 94
    return [AATOAU * v for v in vals]


def lebedev():
    """{size: [[kind, a, b, v], ...]} in the order the reference calls its generators."""
    src = _strip(open(os.path.join(REF, "src/solv/lebedev.f90")).read())
    m = re.search(r"gridSize\(32\)\s*=\s*\[(.*?)\]", src, re.S)
    sizes = [int(t) for t in re.findall(r"\d+", m.group(1).replace("&", " "))]
    grids = {}
    for m in re.finditer(r"subroutine ld(\d{4})\(x, w, n\)(.*?)end subroutine", src, re.S):
        size = int(m.group(1))
        cur = {"a": 0.0, "b": 0.0, "v": 0.0}
        gens = []
        for line in m.group(2).splitlines():
            s = line.strip()
            a = re.match(r"([abv])\s*=\s*(" + NUM.pattern + r")$", s)
            if a:
                cur[a.group(1)] = _num(a.group(2))
                continue
            c = re.match(r"call genOh(\d)\(", s)
            if c:
                kind = int(c.group(1))
                gens.append([kind, cur["a"] if kind >= 4 else 0.0, cur["b"] if kind == 6 else 0.0, cur["v"]])
        npts = sum({1: 6, 2: 12, 3: 8, 4: 24, 5: 24, 6: 48}[g[0]] for g in gens)
        if npts != size:
            raise ValueError(f"ld{size:04d}: generators give {npts} points")
        grids[size] = gens
    assert sorted(grids) == sizes, "every listed grid size needs its generator table"
    return sizes, grids


def c_double(x):
    return repr(float(x)) if np.isfinite(x) else "0.0"


def write_inc(path, gbsa, alpb, vdw, sizes, grids):
    L = ["// Generated by oracle/gen_solvation.py from the reference's solvation tables; do not edit.",
         "// GBSA / ALPB parameter sets for GFN2-xTB (src/solv/model.f90:94-106, include/param_*.fh),",
         "// D3 van der Waals radii in Bohr (src/param/vdwradd3.f90:37) and the Lebedev-Laikov grid",
         "// generators (src/solv/lebedev.f90).",
         "#pragma once",
         "namespace xg { namespace solvdata {",
         "struct ParamSet {",
         "    const char* solvent;",
         "    int alpb;   // 0: GBSA set (Still kernel), 1: ALPB set (P16 kernel)",
         "    double epsv, smass, rhos, c1, rprobe, gshift, soset, alpha;",
         "    double gamscale[94], sx[94], tmp[94];",
         "};"]
    sets = [(k, 0, v) for k, v in sorted(gbsa.items())] + [(k, 1, v) for k, v in sorted(alpb.items())]
    L.append(f"constexpr int NSETS = {len(sets)};")
    L.append("static const ParamSet SETS[NSETS] = {")
    for name, flag, p in sets:
        sc = ", ".join(c_double(p[k]) for k in SCALARS)
        arrs = ",\n     ".join("{" + ", ".join(c_double(x) for x in p[k]) + "}" for k in ("gamscale", "sx", "tmp"))
        L.append(f'    {{"{name}", {flag}, {sc},\n     {arrs}}},')
    L.append("};")
    L.append("static const double VDW_RAD_D3[94] = {" + ", ".join(c_double(x) for x in vdw) + "};")
    L.append(f"constexpr int NGRIDS = {len(sizes)};")
    L.append("static const int GRID_SIZE[NGRIDS] = {" + ", ".join(str(s) for s in sizes) + "};")
    offs, flat = [], []
    for s in sizes:
        offs.append(len(flat))
        flat.extend(grids[s])
    offs.append(len(flat))
    L.append("static const int GRID_GEN_OFFSET[NGRIDS + 1] = {" + ", ".join(str(o) for o in offs) + "};")
    L.append("// per generator: orbit kind (1..6), a, b, weight")
    L.append(f"static const double GRID_GEN[{len(flat)}][4] = {{")
    for g in flat:
        L.append("    {" + ", ".join([str(g[0]) + ".0"] + [c_double(x) for x in g[1:]]) + "},")
    L.append("};")
    L.append("}}  // namespace xg::solvdata")
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def main():
    gbsa = parameter_sets("gfn2_", "gbsa")
    alpb = parameter_sets("gfn2_alpb_", "alpb")
    vdw = vdw_rad_d3()
    sizes, grids = lebedev()
    out = {"source": "reference include/param_{gbsa,alpb}_*.fh, src/param/vdwradd3.f90, src/solv/lebedev.f90",
           "gbsa": gbsa, "alpb": alpb, "vdw_rad_d3": vdw,
           "lebedev_sizes": sizes, "lebedev": {str(k): v for k, v in grids.items()}}
    with open(os.path.join(REPO, "xtb_gb300", "data", "solvation_params.json"), "w") as f:
        json.dump(out, f, indent=0)
    write_inc(os.path.join(REPO, "xtb_gb300", "csrc", "solvation_params.inc"), gbsa, alpb, vdw, sizes, grids)
    print(f"{len(gbsa)} GBSA sets, {len(alpb)} ALPB sets, {len(sizes)} Lebedev grids")


if __name__ == "__main__":
    main()
