"""The Fortran ISO_C_BINDING module (include/xtb_gb300.f90) against the C headers and the library
(CPU only; no Fortran compiler is needed): every function the headers declare has an interface
with the same name and number of arguments, every dummy argument is declared, and the library
exports every bound name."""
import os
import re

import pytest

from xtb_gb300 import interface as X

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def c_prototypes():
    """name -> number of parameters, for every function declared in include/*.h"""
    out = {}
    for h in ("xtb.h", "xtb_gb300.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"#[^\n]*", "", src)
        for m in re.finditer(r"\b(xtb(?:gb)?_\w+)\s*\(([^;{}]*?)\)\s*;", src, flags=re.S):
            name, params = m.group(1), " ".join(m.group(2).split())
            out[name] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def fortran_interfaces():
    """bound C name -> (Fortran name, dummy arguments, declaration lines of the body)"""
    src = open(os.path.join(ROOT, "include", "xtb_gb300.f90")).read()
    src = re.sub(r"&\s*\n\s*", " ", src)                       # join continuation lines
    src = "\n".join(line.split("!")[0] for line in src.splitlines())
    out = {}
    pat = re.compile(r"^\s*(?:[\w(), ]+?\s+)?(subroutine|function)\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)"
                     r"(.*?)^\s*end\s+(subroutine|function)", re.M | re.S)
    for m in pat.finditer(src):
        kind, fname, args, cname, body, endkind = m.groups()
        assert kind == endkind, fname
        dummies = [a.strip() for a in args.split(",") if a.strip()]
        out[cname] = (fname, dummies, body)
    return out, src


def test_every_declared_function_has_an_interface():
    c = c_prototypes()
    f, _ = fortran_interfaces()
    assert len(c) >= 80
    missing = sorted(set(c) - set(f))
    extra = sorted(set(f) - set(c))
    assert not missing, missing
    assert not extra, extra


def test_interfaces_match_the_prototypes():
    c = c_prototypes()
    f, _ = fortran_interfaces()
    for cname, (fname, dummies, body) in f.items():
        assert fname == cname, (fname, cname)
        assert len(dummies) == c[cname], (cname, dummies, c[cname])
        declared = set(re.findall(r"::\s*([\w ,()*]+)", body))
        names = set()
        for d in declared:
            names |= {re.sub(r"\(.*", "", x).strip().lower() for x in re.split(r",(?![^(]*\))", d)}
        for a in dummies:
            assert a.lower() in names, (cname, a)


def test_public_names_and_imports():
    f, src = fortran_interfaces()
    public = set()
    for line in re.findall(r"^\s*public\s*::\s*(.*)$", src, flags=re.M):
        public |= {x.strip() for x in line.split(",") if x.strip()}
    assert public == {v[0] for v in f.values()}
    for cname, (_, _, body) in f.items():
        imp = re.search(r"import\s*::\s*(.*)", body)
        used = set(re.findall(r"\b(c_ptr|c_int|c_double|c_char|c_long_long)\b", body.split("\n", 2)[-1] if imp else body))
        have = {x.strip() for x in imp.group(1).split(",")} if imp else set()
        assert used <= have, (cname, used - have)


def test_library_exports_every_bound_name():
    try:
        lib = X.load_library()
    except X.XTBException as e:
        pytest.skip(str(e))
    f, _ = fortran_interfaces()
    missing = [n for n in f if not hasattr(lib, n)]
    assert not missing, missing
