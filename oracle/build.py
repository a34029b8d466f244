"""Build the oracle's C++ restatement into ``oracle/_build/`` (test infrastructure).

Two shared libraries are made from ``tetra_weights.cpp``:

* ``liboracle_weights.so`` — portable atan/log (bit-identical to the GPU);
* ``liboracle_weights_libm.so`` — the C library's atan/log, used to measure
  how far the reference's own formulas spread under a different libm.

Both use ``-O3 -ffp-contract=off -fopenmp`` and no ISA-specific flags, so the
same recipe builds on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "tetra_weights.cpp")
HDR = os.path.join(HERE, "..", "pygw_gb300", "csrc", "fp64_math.h")

TARGETS = {
    "liboracle_weights.so": [],
    "liboracle_weights_libm.so": ["-DORACLE_LIBM"],
}


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False):
    os.makedirs(BUILD, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    procs = []
    for name, extra in TARGETS.items():
        out = os.path.join(BUILD, name)
        if not force and not _stale(out, [SRC, HDR, __file__]):
            continue
        cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               *extra, SRC, "-o", out + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd), out))
    for p, out in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed for {out}")
        os.replace(out + ".tmp", out)
    return {n: os.path.join(BUILD, n) for n in TARGETS}


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
