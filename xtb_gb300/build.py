"""In-tree build of libxtb_gb300.so (sm_103a) with nvcc; no CMake, no PyTorch.

Usage: ``python -m xtb_gb300.build`` (or ``__graft_entry__.build()``).  Each
translation unit is compiled in parallel, then linked into a shared library
next to this file.  Re-running only recompiles changed sources.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libxtb_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cpp", "host_model.cpp", "engine.cu", "gfn2_kernels.cu", "integrals.cu", "linalg.cu", "noalloc.cu", "batch.cu", "batch_integrals.cu", "batch_runner.cpp", "serve.cpp", "splitgemm.cu", "tune.cu", "solvation.cu"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the GB300 engine needs the CUDA toolkit to build")
    return exe


def _needs(src, obj):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    for h in ("xtb.h", "xtb_gb300.h"):
        deps.append(os.path.join(os.path.dirname(HERE), "include", h))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    if not _needs(path, obj):
        return obj, ""
    cmd = [nvcc()] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        results = list(ex.map(_compile, SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
