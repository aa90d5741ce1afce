"""Build recipe for the CPU oracle (test infrastructure only).

* ``liboracle.so``   -- the plain-C restatement in ``mcoracle.c``; builds anywhere
  gcc is present (this container and the GPU host alike).
* ``_ref/libref.so`` -- the reference engine compiled from its own sources under
  ``/root/reference/engine`` together with ``ref_driver.c`` (a small C driver
  written here).  It exists only where the reference tree is mounted and is used
  to cross-check the restatement; nothing on the GPU host needs it.

Both are built with -ffp-contract=off and without -ffast-math: the reference's
results depend on unfused IEEE float/double arithmetic.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_ROOT = os.environ.get("MCGEN_REFERENCE_ROOT", "/root/reference")  # the reference source tree
CFLAGS = ["-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared"]


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(verbose: bool = False) -> str:
    out = os.path.join(HERE, "liboracle.so")
    src = [os.path.join(HERE, "mcoracle.c")]
    if _stale(out, src + [os.path.join(HERE, "mcoracle.h")]):
        cmd = ["gcc", *CFLAGS, *src, "-o", out + ".tmp", "-lm"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.check_call(cmd)
        os.replace(out + ".tmp", out)
    return out


def build_reference(verbose: bool = False) -> str | None:
    """Compile the reference engine's CPU path (engine/cuda/mcg_host.c + headers) with our driver."""
    host_c = os.path.join(REFERENCE_ROOT, "engine", "cuda", "mcg_host.c")
    if not os.path.exists(host_c):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libref.so")
    drv = os.path.join(HERE, "ref_driver.c")
    if _stale(out, [drv]):
        cmd = ["gcc", *CFLAGS, "-I", os.path.join(REFERENCE_ROOT, "engine", "cuda"),
               "-I", os.path.join(REFERENCE_ROOT, "engine"), host_c, drv, "-o", out + ".tmp", "-lm"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.check_call(cmd)
        os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_reference(verbose=True))
