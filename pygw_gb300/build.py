"""Build ``libpygw_gb300.so`` in-tree (``pygw_gb300/_build/``) with nvcc for sm_103a.

Each ``.cu`` under ``csrc/`` is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``; the weight kernel
additionally gets ``-fmad=false`` so its arithmetic matches the CPU oracle bit
for bit (every fused multiply-add in it is written explicitly).  The library
links the shared CUDA runtime so it shares one runtime with PyTorch.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpygw_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# per-file extra flags
SOURCES = {
    "weights.cu": ["-fmad=false"],
    "chi0_f64.cu": [],
    "eps_f64.cu": [],
    "launches.cu": [],
    "chi0_mixed.cu": [],
    "eps_mixed.cu": [],
    "synth.cu": [],
    "selfc.cu": [],
}


def nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _deps():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    out.append(os.path.abspath(__file__))
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    cc = nvcc()
    common = [*ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", CSRC]
    procs = []
    objs = []
    for src, extra in SOURCES.items():
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if not force and not _stale(obj, deps):
            continue
        cmd = [cc, *common, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), src))
    failed = []
    for p, src in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(f"--- {s}\n{o}" for s, o in failed))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
