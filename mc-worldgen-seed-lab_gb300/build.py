"""Build recipe of the CUDA library libmcgen_gb300.so (sm_103a), in-tree.

Every translation unit is compiled by nvcc for sm_103a only, with IEEE float/double semantics kept
intact: --fmad=false (no contraction of a*b+c), IEEE division and square root, no flush-to-zero, and
-ffp-contract=off for the host compiler.  The translation units build in parallel, then link into one
shared library next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmcgen_gb300.so")
# the reference library's name, for C callers that link with -lmcgen: a symbolic link to LIB (no soname is
# set, so a program linked against either name records that name and loads it at run time)
DROPIN = os.path.join(HERE, "libmcgen.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
                  "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math,-O2", "-I", CSRC, "-I", INCLUDE]
SOURCES = ["kernels.cu", "pipes.cu", "api.cpp", "world.cpp", "prof.cpp", "noalloc.cu", "fused.cu", "selfcheck.cu", "batch.cu",
           "plan.cpp", "server.cpp", "search.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".cu", ".cpp"))]
    out += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return out + [os.path.abspath(__file__)]


def _dropin_link() -> None:
    if os.path.islink(DROPIN) and os.readlink(DROPIN) == os.path.basename(LIB):
        return
    if os.path.lexists(DROPIN):
        os.remove(DROPIN)
    os.symlink(os.path.basename(LIB), DROPIN)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    if os.path.exists(LIB) and not ptxas_info:
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            _dropin_link()
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def one(src: str) -> str:
        obj = os.path.join(BUILD, src + ".o")
        cmd = [cc, *NVFLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if ptxas_info and src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if (verbose or ptxas_info) and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart=static"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    _dropin_link()
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
