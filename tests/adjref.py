"""ctypes binding of the CPU reference adjoint (tests/cpp/adjoint_ref.cpp), test-only."""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def lib():
    global _lib
    if _lib is None:
        out = os.path.join(tempfile.gettempdir(), f"adjref_{os.getpid()}.so")
        src = os.path.join(HERE, "cpp", "adjoint_ref.cpp")
        subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-o", out, src], check=True)
        L = ctypes.CDLL(out)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        i, d = ctypes.c_int, ctypes.c_double
        L.adjref_run.argtypes = [i, i, d, d, d, i, i, d, dp, dp, dp, dp, i, ip, ip, dp, dp, dp, dp, dp]
        L.adjref_run.restype = ctypes.c_double
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def run(Nx, Ny, h, hu, hv, B, steps, dt, gi, gj, obs, grads=True, Lx=1.0, Ly=1.0,
        g=9.80665, bc=0):
    gi = np.ascontiguousarray(gi, dtype=np.int32)
    gj = np.ascontiguousarray(gj, dtype=np.int32)
    obs = np.ascontiguousarray(obs, dtype=np.float64)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (h, hu, hv, B)]
    out = [np.zeros_like(arrs[0]) for _ in range(4)] if grads else [None] * 4
    ip = ctypes.POINTER(ctypes.c_int)
    J = lib().adjref_run(Nx, Ny, Lx, Ly, g, bc, steps, dt, *(_p(a) for a in arrs), len(gi),
                         gi.ctypes.data_as(ip), gj.ctypes.data_as(ip), _p(obs),
                         *(_p(a) for a in out))
    return (J, *out) if grads else J
