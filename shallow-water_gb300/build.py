"""Builds libswe_gb300.so in-tree with nvcc for sm_103a (GB300).

Each translation unit compiles in parallel with its own flags, then one link.
The FP64 drop-in (swe_fp64.cu) and the modular solver (swe_modular.cu) are compiled
with --fmad=false so that no a*b+c is fused: that keeps their arithmetic bitwise equal
to the reference's CPU solvers.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libswe_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]

# source -> extra flags
UNITS = {
    "swe_fp64.cu": ["--fmad=false"],
    "swe_modular.cu": ["--fmad=false"],
    "swe_fp32.cu": [],
    "swe_reduce.cu": [],
    "swe_ensemble.cu": [],
    "swe_adjoint.cu": [],
    "swe_selftest.cu": [],
    "swe_output.cu": [],
    "swe_ncfile.cpp": [],
    "swe_api.cu": [],
    "swe_slabs.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libswe_gb300.so")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".map"))]
    headers.append(os.path.join(HERE, "..", "include", "swe_gb300.h"))
    objs, procs = [], []
    cc = nvcc()
    for src, extra in UNITS.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [cc, *ARCH, *COMMON, *extra, "-c", s, "-o", o]
            log = open(o + ".log", "w")
            procs.append((cmd, subprocess.Popen(cmd, stdout=log, stderr=subprocess.STDOUT), o))
    for cmd, p, o in procs:
        if p.wait() != 0:
            sys.stderr.write(open(o + ".log").read())
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
        if verbose:
            sys.stderr.write(open(o + ".log").read())
    if force or _stale(LIB, objs):
        # the C ABI only (swe_*); the kernels' C++ launchers stay internal
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart",
               "-Xlinker", "--version-script=" + os.path.join(CSRC, "swe_gb300.map")]
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
