"""ctypes binding of the reference's own solver built by ``make ref`` (test infrastructure).

Available only where the reference sources were present at build time; callers
skip when :func:`available` is False.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_dir() -> str:
    """Where the reference's sources lie: SWE_REFERENCE_DIR, else the oracle recipe's
    default (``make -C oracle print-ref``)."""
    d = os.environ.get("SWE_REFERENCE_DIR")
    if d:
        return d
    try:
        return subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True,
                              text=True, check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return ""
LIBS = {
    "g980665": os.path.join(HERE, "_ref", "libswe_ref.so"),
    "g981": os.path.join(HERE, "_ref", "libswe_ref_g981.so"),
}
SOLVER_HPC = 0
SOLVER_OMP = 1

_libs = {}


def available(variant="g980665") -> bool:
    return os.path.exists(LIBS[variant])


def lib(variant="g980665"):
    if variant not in _libs:
        L = ctypes.CDLL(LIBS[variant])
        dp = ctypes.POINTER(ctypes.c_double)
        i, d = ctypes.c_int, ctypes.c_double
        L.ref_run.argtypes = [i, i, d, d, d, i, i, i, d, dp, dp, dp, dp, dp, dp]
        L.ref_run.restype = ctypes.c_int
        L.ref_stable_dt.argtypes = [i, i, d, d, d, dp, dp, dp]
        L.ref_stable_dt.restype = ctypes.c_double
        L.ref_gravity.argtypes = []
        L.ref_gravity.restype = ctypes.c_double
        L.ref_modular_run.argtypes = [i, i, d, d, d, i, i, i, i, d, dp, dp, dp, dp]
        L.ref_modular_run.restype = ctypes.c_int
        L.ref_modular_stable_dt.argtypes = [i, i, d, d, d, dp, dp, dp, dp]
        L.ref_modular_stable_dt.restype = ctypes.c_int
        _libs[variant] = L
    return _libs[variant]


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def run(Nx, Ny, h, hu, hv, B, steps, dt_fixed=0.0, Lx=1.0, Ly=1.0, cfl=0.45, bc=0,
        solver=SOLVER_HPC, variant="g980665"):
    """Runs the reference; returns (h, hu, hv, dts, t, status) on copies."""
    h, hu, hv = (np.array(a, dtype=np.float64, order="C", copy=True) for a in (h, hu, hv))
    B = np.ascontiguousarray(B, dtype=np.float64)
    dts = np.zeros(max(steps, 1))
    t = ctypes.c_double(0.0)
    st = lib(variant).ref_run(Nx, Ny, Lx, Ly, cfl, bc, solver, steps, dt_fixed, _p(h), _p(hu),
                              _p(hv), _p(B), _p(dts), ctypes.byref(t))
    return h, hu, hv, dts[:steps], t.value, st


def stable_dt(Nx, Ny, h, hu, hv, Lx=1.0, Ly=1.0, cfl=0.45, variant="g980665") -> float:
    return lib(variant).ref_stable_dt(Nx, Ny, Lx, Ly, cfl, _p(h), _p(hu), _p(hv))


def gravity(variant="g980665") -> float:
    return lib(variant).ref_gravity()


def modular_run(Nx, Ny, recon, riemann, bathy, h, hu, hv, B, steps, dt, Lx=1.0, Ly=1.0,
                cfl=0.45, variant="g980665"):
    """The reference's SerialSolver on copies (recon 0/1, riemann 0/1/2 as
    oracle.port.RECON / RIEMANN); returns (h, hu, hv, status)."""
    h, hu, hv = (np.array(a, dtype=np.float64, order="C", copy=True) for a in (h, hu, hv))
    B = np.ascontiguousarray(B, dtype=np.float64)
    st = lib(variant).ref_modular_run(Nx, Ny, Lx, Ly, cfl, recon, riemann, int(bool(bathy)),
                                      steps, dt, _p(h), _p(hu), _p(hv), _p(B))
    return h, hu, hv, st


def modular_stable_dt(Nx, Ny, h, hu, hv, Lx=1.0, Ly=1.0, cfl=0.45, variant="g980665"):
    out = ctypes.c_double(0.0)
    st = lib(variant).ref_modular_stable_dt(Nx, Ny, Lx, Ly, cfl, _p(h), _p(hu), _p(hv),
                                            ctypes.byref(out))
    return out.value, st
