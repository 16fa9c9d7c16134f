"""In-tree build of libsfci_gb300.so and the native ``sfci`` driver binary.

nvcc compiles the CUDA translation units for sm_103a only; the host C++ units
go through g++.  Objects and outputs land in ``sfci_gb300/_build`` (ignored by
git).  Each unit is rebuilt only when it or a header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsfci_gb300.so")
EXE = os.path.join(BUILD, "sfci")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_UNITS = ["prims.cu", "spmspv.cu", "vecops.cu", "noalloc.cu", "subspace.cu", "mlp.cu"]
CXX_UNITS = ["abi.cpp", "solver.cpp", "ham.cpp", "vecio.cpp"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    raise RuntimeError("CUDA toolkit not found (nvcc missing)")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "sfci_gb300.h"))
    return hs


def _stale(src: str, obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src, *deps])


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile (if needed) and return the path of libsfci_gb300.so."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    deps = _headers()
    inc = ["-I" + os.path.join(cuda, "include"), "-I" + CSRC]
    jobs = []
    objs = []
    for u in CU_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if force or _stale(src, obj, deps):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
                         *inc, "-c", src, "-o", obj])
    for u in CXX_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if force or _stale(src, obj, deps):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", *inc, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                if o.strip():
                    print(o)
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    main_src = os.path.join(CSRC, "sfci_main.cpp")
    if os.path.exists(main_src) and (force or not os.path.exists(EXE) or _stale(main_src, EXE, deps + [LIB])):
        _run(["g++", "-std=c++17", "-O2", *inc, main_src, "-o", EXE, "-L" + BUILD, "-lsfci_gb300",
              "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
