"""Generate tests/golden/gfn2_reference.json from the reference's own GFN2 tests.

Reads (as text) test/unit/test_gfn2.f90 and test/api/c_api_example.c of the
reference tree and extracts, for each known-answer case, the geometry and the
values the reference asserts, with the tolerance it asserts them at:

* ``scc``   test_gfn2.f90:48-170   water, zero-charge guess, energy parts, charges, multipoles
* ``api``   test_gfn2.f90:172-235  propyne C3H4, EEQ guess, energy, gap, gradient
* ``pcem``  test_gfn2.f90:383-457  (H2O)4 cluster without point charges, energy, gap, gradient
* ``pcem_charges``, ``pcem_point``  test_gfn2.f90:459-520  (H2O)2 in the field of the other two
            waters as six external charges, with GFN2 hardnesses and with gamma = 999 (bare point
            charges): energy, gap, gradient, point-charge gradient
* ``capi``  c_api_example.c:38-112 propyne through the C ABI: energy, q[5], dipole, wbo
* ``capi_pc`` c_api_example.c:298-410 the same dimer through xtb_setExternalCharges: energy,
            gradient and point-charge gradient
* ``gbsa``  test_gfn2.f90:237-308  11-atom molecule in water (GBSA, Still kernel): energy, gap,
            gradient
* ``salt``  test_gfn2.f90:310-381  8-atom molecule in CH2Cl2 with 1 mM salt (ion radius 1 A)
* ``capi_gbsa``, ``capi_alpb`` c_api_example.c:114-163 propyne in water through xtb_setSolvent
            ("gbsa", then "alpb"), each started from the previous result's wavefunction
* ``mindless_solvation`` test_gfn2.f90:745-828 mindless01-10 in ten solvents, every second one
            with the ALPB correction (Still kernel)

Usage: python tests/golden/make_golden.py [reference_root]
"""
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gfn2_reference.json")
NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eEdD][-+]?\d+)?"


SYMBOLS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br "
           "Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er "
           "Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn").split()


def fnum(t):
    return float(t.replace("_wp", "").replace("d", "e").replace("D", "e"))


def sub(src, name):
    a = src.index(f"subroutine {name}(")
    b = src.index(f"end subroutine {name}", a)
    return src[a:b]


def array(block, decl):
    m = re.search(decl + r"[^=]*=\s*(?:reshape\(\s*)?\[?&?(.*?)\]", block, re.S)
    body = re.sub(r"!.*", "", m.group(1)).replace("&", " ")
    return [fnum(t) for t in re.findall(NUM + r"(?:_wp)?", body)]


def checks(block):
    out = []
    for m in re.finditer(r"call check_\(error,\s*((?:[^,(\n]|\([^)\n]*\))+),\s*(" + NUM + r")_wp(?:,\s*thr=([^)]+))?\)", block):
        out.append({"expr": m.group(1).strip(), "value": fnum(m.group(2)), "thr": m.group(3)})
    return out


def main():
    src = open(os.path.join(REF, "test/unit/test_gfn2.f90")).read()
    cases = {}
    for key, name in (("scc", "test_gfn2_scc"), ("api", "test_gfn2_api"), ("pcem", "test_gfn2_pcem_api")):
        blk = sub(src, name)
        if key == "pcem":
            blk = blk[:blk.index("! reset")]
        at = [int(v) for v in array(blk, r"integer, parameter :: at\(nat\)")]
        xyz = array(blk, r"real\(wp\),parameter :: xyz\(3,nat\)")
        thr = {}
        for m in re.finditer(r"real\(wp\),parameter :: (thr2?)\s*=\s*(" + NUM + r")_wp", blk):
            thr[m.group(1)] = fnum(m.group(2))
        cs = checks(blk)
        for c in cs:
            t = c["thr"]
            if t is None:
                c["thr"] = 1e-15
            elif t in thr:
                c["thr"] = thr[t]
            elif "*" in t:
                base, fac = t.split("*")
                c["thr"] = thr[base.strip()] * float(fac)
            else:
                c["thr"] = fnum(t)
        maxiter = int(re.search(r"maxiter\s*=\s*(\d+)", blk).group(1))
        cases[key] = {"numbers": at, "positions": xyz, "checks": cs, "maxiter": maxiter,
                      "guess": "zero" if key == "scc" else "eeq"}
        if key == "pcem":
            # the second half: molecule = first two waters, the other two as external charges
            full = sub(src, name)
            rest = full[full.index("! reset"):]
            q = array(full, r"real\(wp\),parameter :: q\(nat2\)")
            gam = array(full, r"real\(wp\),parameter :: gam\(nat2\)")
            nat2 = len(at) // 2
            parts = rest.split("! reset")
            for pkey, part, g in (("pcem_charges", parts[1], gam), ("pcem_point", parts[2], [999.0] * nat2)):
                pcs = []
                for c in checks(part):
                    c["thr"] = thr["thr"]
                    pcs.append(c)
                cases[pkey] = {"numbers": at[:nat2], "positions": xyz[:3 * nat2], "pc_charges": q,
                               "pc_positions": xyz[3 * nat2:], "pc_gam": g, "checks": pcs,
                               "maxiter": maxiter, "guess": "eeq"}
    capi = open(os.path.join(REF, "test/api/c_api_example.c")).read()
    first = capi[capi.index("testFirst"):capi.index("testSecond")]
    m = re.search(r"double const coord\[[^\]]*\]\s*=\s*\{(.*?)\};", first, re.S)
    coord = [fnum(t) for t in re.findall(NUM, m.group(1))]
    m = re.search(r"int const attyp\[7\]\s*=\s*\{(.*?)\};", first, re.S)
    at = [int(t) for t in re.findall(r"\d+", m.group(1))]
    cks = []
    for m in re.finditer(r"check\((\w+(?:\[\d+\])?),\s*(" + NUM + r"),\s*(" + NUM + r")", first):
        cks.append({"expr": m.group(1), "value": fnum(m.group(2)), "thr": fnum(m.group(3))})
    cases["capi"] = {"numbers": at, "positions": coord, "checks": cks[:4], "maxiter": 30, "guess": "eeq"}
    # numerical Hessian of the same molecule (xtb_hessian, default step, fresh results object):
    # hess[i] is element i of the flattened 3N x 3N matrix
    hk = [c for c in cks if c["expr"].startswith("hess[")]
    natsq = len(at) * len(at)
    m = re.search(r"check\(hess\[\(9\*natsq\)-1\],\s*(" + NUM + r"),\s*(" + NUM + r")", first)
    hk.append({"expr": f"hess[{9 * natsq - 1}]", "value": fnum(m.group(1)), "thr": fnum(m.group(2))})
    cases["capi_hessian"] = {"numbers": at, "positions": coord, "checks": hk, "maxiter": 250, "guess": "eeq",
                             "step": 0.005}
    # testSecond: the water dimer with six external charges through xtb_setExternalCharges
    second = capi[capi.index("int testSecond"):]
    second = second[:second.index("error:")]

    def carr(name):
        m = re.search(r"\b" + name + r"\[[^\]]*\]\s*=\s*\{(.*?)\};", second, re.S)
        return [fnum(t) for t in re.findall(NUM, m.group(1))]

    pck = []
    for m in re.finditer(r"check\((\w+\[[^\]]+\]|\w+),\s*(" + NUM + r"),\s*(" + NUM + r")", second):
        expr = m.group(1)
        mi = re.fullmatch(r"(\w+)\[(\d+) \+ (\d+) \* 3\]", expr)
        if mi:
            expr = f"{mi.group(1)}[{int(mi.group(2)) + 3 * int(mi.group(3))}]"
        pck.append({"expr": expr, "value": fnum(m.group(2)), "thr": fnum(m.group(3))})
    cases["capi_pc"] = {"numbers": [int(v) for v in carr("attyp")], "positions": carr("coord"),
                        "pc_charges": carr("pc"), "pc_positions": carr("pccoord"),
                        "pc_numbers": [int(v) for v in carr("numbers")], "checks": pck, "maxiter": 250,
                        "guess": "eeq"}
    # mindless01-10 (test_gfn2.f90:667-742, geometries from test/unit/molstock.f90): energy,
    # gradient norm and HOMO-LUMO gap at 1e-8 after a default single point from the EEQ guess
    blk = sub(src, "test_gfn2_mindless_basic")
    ref = {}
    for key in ("ref_energies", "ref_gnorms", "ref_hlgaps"):
        m = re.search(key + r"\(10\)\s*=[\s&]*\[(.*?)\]", blk, re.S)
        ref[key] = [fnum(t) for t in re.findall(NUM, m.group(1))]
    stock = open(os.path.join(REF, "test/unit/molstock.f90")).read()
    mols = []
    for i in range(1, 11):
        name = f"mindless{i:02d}"
        a = stock.index(f"subroutine {name}(mol)")
        b = stock.index(f"end subroutine {name}", a)
        body = stock[a:b]
        syms = re.findall(r'"([A-Za-z]{1,2})\s*"', body[body.index("sym(nat)"):body.index("xyz(3, nat)")])
        xyz = [fnum(t) for t in re.findall(NUM + r"(?=_wp)", body[body.index("xyz(3, nat)"):])]
        mols.append({"name": name, "numbers": [SYMBOLS.index(x.capitalize()) + 1 for x in syms],
                     "positions": xyz, "energy": ref["ref_energies"][i - 1], "gnorm": ref["ref_gnorms"][i - 1],
                     "hl_gap": ref["ref_hlgaps"][i - 1], "thr": 1e-8})
    cases["mindless"] = mols
    # implicit solvation
    for key, name in (("gbsa", "test_gfn2gbsa_api"), ("salt", "test_gfn2salt_api")):
        blk = sub(src, name)
        at = [int(v) for v in array(blk, r"integer, parameter :: at\(nat\)")]
        xyz = array(blk, r"real\(wp\),parameter :: xyz\(3,nat\)")
        thr = fnum(re.search(r"real\(wp\),parameter :: thr\s*=\s*(" + NUM + r")_wp", blk).group(1))
        cs = []
        for c in checks(blk):
            c["thr"] = thr if c["thr"] in (None, "thr") else fnum(c["thr"])
            cs.append(c)
        solvent = re.search(r'solvent\s*=\s*[\'"](\w+)[\'"]', blk).group(1)
        add = blk[blk.index("call addSolvationModel"):]
        add = add[:add.index("call calc%singlepoint")]
        assert "alpb=.false." in add and "kernel=gbKernel%still" in add, add
        case = {"numbers": at, "positions": xyz, "checks": cs,
                "maxiter": int(re.search(r"maxiter\s*=\s*(\d+)", blk).group(1)), "guess": "eeq",
                "solvent": solvent, "kernel": "still", "alpb": False}
        if key == "salt":
            m = re.search(r"ionRad=(" + NUM + r")_wp\*aatoau, ionStrength=(" + NUM + r")_wp", add)
            case["ion_rad_angstrom"] = fnum(m.group(1))
            case["ion_strength"] = fnum(m.group(2))
        cases[key] = case
    blk = sub(src, "test_gfn2_mindless_solvation")
    ref = {}
    for key in ("ref_energies", "ref_gnorms", "ref_hlgaps"):
        m = re.search(key + r"\(10\)\s*=[\s&]*\[(.*?)\]", blk, re.S)
        ref[key] = [fnum(t) for t in re.findall(NUM, m.group(1))]
    m = re.search(r"solvents\(10\)\s*=\s*\[character\(len=20\)\s*::(.*?)\]", blk, re.S)
    solvents = re.findall(r'"(\w+)"', m.group(1))
    assert "alpb=mod(iMol, 2)==0, kernel=gbKernel%still" in blk
    cases["mindless_solvation"] = [
        {"name": mols[i]["name"], "numbers": mols[i]["numbers"], "positions": mols[i]["positions"],
         "solvent": solvents[i], "kernel": "still", "alpb": (i + 1) % 2 == 0,
         "energy": ref["ref_energies"][i], "gnorm": ref["ref_gnorms"][i], "hl_gap": ref["ref_hlgaps"][i],
         "thr": 1e-8} for i in range(10)]
    for key, start, stop, model in (("capi_gbsa", "// GBSA", "// ALPB", "gbsa"),
                                    ("capi_alpb", "// ALPB", "// COSMO", "alpb")):
        part = first[first.index(start):first.index(stop)]
        assert f"NULL, NULL, NULL, {model});" in part
        cks = [{"expr": m.group(1), "value": fnum(m.group(2)), "thr": fnum(m.group(3))}
               for m in re.finditer(r"check\((\w+(?:\[\d+\])?),\s*(" + NUM + r"),\s*(" + NUM + r")", part)]
        cases[key] = {"numbers": cases["capi"]["numbers"], "positions": cases["capi"]["positions"],
                      "checks": cks, "maxiter": 30, "guess": "eeq", "solvent": "h2o", "model": model,
                      "warm_start_from": "capi" if model == "gbsa" else "capi_gbsa"}
    json.dump(cases, open(OUT, "w"), indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
