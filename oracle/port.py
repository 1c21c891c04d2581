"""ctypes binding of the C restatement of the reference hot path (test infrastructure).

Functions mirror ``oracle/swe_oracle.h``.  Arrays are full ghosted float64
``(Nx + 4, Ny + 4)`` row-major grids, i = x (slow), j = y (contiguous).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libswe_oracle.so")

BC_REFLECTING = 0
BC_TRANSMISSIVE = 1
G_REFERENCE = 9.80665  # include/constants.hpp:4


class _Grid(ctypes.Structure):
    _fields_ = [
        ("Nx", ctypes.c_int),
        ("Ny", ctypes.c_int),
        ("Lx", ctypes.c_double),
        ("Ly", ctypes.c_double),
        ("g", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("bc", ctypes.c_int),
        ("threads", ctypes.c_int),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
    ]


_lib = None


def build() -> str:
    """Compiles the restatement with ``make port`` (no-op when up to date)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        gp = ctypes.POINTER(_Grid)
        L.swe_oracle_run.argtypes = [gp, ctypes.c_int, ctypes.c_double, dp, dp, dp, dp, dp, dp]
        L.swe_oracle_run.restype = ctypes.c_int
        L.swe_oracle_ws_create.argtypes = [gp]
        L.swe_oracle_ws_create.restype = ctypes.c_void_p
        L.swe_oracle_ws_destroy.argtypes = [ctypes.c_void_p]
        L.swe_oracle_ws_destroy.restype = None
        L.swe_oracle_run_ws.argtypes = [gp, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                        dp, dp, dp, dp, dp, dp]
        L.swe_oracle_run_ws.restype = ctypes.c_int
        L.swe_oracle_stage.argtypes = [gp, ctypes.c_int, ctypes.c_double] + [dp] * 10
        L.swe_oracle_stage.restype = ctypes.c_int
        L.swe_oracle_stable_dt.argtypes = [gp, dp, dp, dp]
        L.swe_oracle_stable_dt.restype = ctypes.c_double
        L.swe_oracle_max_wave_speed.argtypes = [gp, dp, dp, dp]
        L.swe_oracle_max_wave_speed.restype = ctypes.c_double
        L.swe_oracle_fill_ghosts.argtypes = [gp, dp, dp, dp]
        L.swe_oracle_fill_ghosts.restype = None
        L.swe_oracle_fill_scalar_ghosts.argtypes = [gp, dp]
        L.swe_oracle_fill_scalar_ghosts.restype = None
        i = ctypes.c_int
        L.swe_oracle_modular_run.argtypes = [gp, i, i, i, i, ctypes.c_double, dp, dp, dp, dp, dp]
        L.swe_oracle_modular_run.restype = ctypes.c_int
        L.swe_oracle_modular_stable_dt.argtypes = [gp, dp, dp, dp, dp]
        L.swe_oracle_modular_stable_dt.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def grid(Nx, Ny, Lx=1.0, Ly=1.0, g=G_REFERENCE, cfl=0.45, bc=BC_REFLECTING, threads=0,
         dx=0.0, dy=0.0):
    return _Grid(Nx, Ny, Lx, Ly, g, cfl, bc, threads, dx, dy)


def run(p: _Grid, h, hu, hv, B, steps, dt_fixed=0.0):
    """Runs ``steps`` SSP-RK3 steps on copies; returns (h, hu, hv, dts, t, status)."""
    h, hu, hv = (np.array(a, dtype=np.float64, order="C", copy=True) for a in (h, hu, hv))
    B = np.ascontiguousarray(B, dtype=np.float64)
    dts = np.zeros(max(steps, 1))
    t = ctypes.c_double(0.0)
    st = lib().swe_oracle_run(ctypes.byref(p), steps, dt_fixed, _p(h), _p(hu), _p(hv), _p(B),
                              _p(dts), ctypes.byref(t))
    return h, hu, hv, dts[:steps], t.value, st


class Workspace:
    """Work buffers for repeated in-place runs on one grid (allocation kept out of timing)."""

    def __init__(self, p: _Grid):
        self.p = p
        self.ws = lib().swe_oracle_ws_create(ctypes.byref(p))
        if not self.ws:
            raise MemoryError("swe_oracle_ws_create failed")

    def run_inplace(self, h, hu, hv, B, steps, dt_fixed=0.0):
        """Advances h, hu, hv in place; returns (dts, t, status)."""
        dts = np.zeros(max(steps, 1))
        t = ctypes.c_double(0.0)
        st = lib().swe_oracle_run_ws(ctypes.byref(self.p), self.ws, steps, dt_fixed, _p(h),
                                     _p(hu), _p(hv), _p(B), _p(dts), ctypes.byref(t))
        return dts[:steps], t.value, st

    def close(self):
        if self.ws:
            lib().swe_oracle_ws_destroy(self.ws)
            self.ws = None

    def __del__(self):
        self.close()


def stage(p: _Grid, stage_no, dt, Un, Us, B):
    """One RK stage; returns (h, hu, hv, status)."""
    out = [np.zeros_like(Us[0]) for _ in range(3)]
    Un = Us if Un is None else Un
    st = lib().swe_oracle_stage(ctypes.byref(p), stage_no, dt, *[_p(np.ascontiguousarray(a)) for a in Un],
                                *[_p(np.ascontiguousarray(a)) for a in Us],
                                _p(np.ascontiguousarray(B)), *[_p(a) for a in out])
    return out[0], out[1], out[2], st


def stable_dt(p: _Grid, h, hu, hv) -> float:
    return lib().swe_oracle_stable_dt(ctypes.byref(p), _p(h), _p(hu), _p(hv))


def max_wave_speed(p: _Grid, h, hu, hv) -> float:
    return lib().swe_oracle_max_wave_speed(ctypes.byref(p), _p(h), _p(hu), _p(hv))


def fill_ghosts(p: _Grid, h, hu, hv):
    lib().swe_oracle_fill_ghosts(ctypes.byref(p), _p(h), _p(hu), _p(hv))


def fill_scalar_ghosts(p: _Grid, a):
    lib().swe_oracle_fill_scalar_ghosts(ctypes.byref(p), _p(a))


RECON = {"PiecewiseConst": 0, "MUSCL": 1}
RIEMANN = {"HLL": 0, "Rusanov": 1, "ROE": 2}


def modular_run(p: _Grid, recon, riemann, bathy, h, hu, hv, B, steps, dt):
    """SerialSolver<ReflectingWalls, recon, riemann, SSPRK3, bathymetry on/off> for
    ``steps`` fixed-dt steps on copies; returns (h, hu, hv, t, status)."""
    h, hu, hv = (np.array(a, dtype=np.float64, order="C", copy=True) for a in (h, hu, hv))
    B = np.ascontiguousarray(B, dtype=np.float64)
    t = ctypes.c_double(0.0)
    st = lib().swe_oracle_modular_run(ctypes.byref(p), RECON.get(recon, recon),
                                      RIEMANN.get(riemann, riemann), int(bool(bathy)), steps, dt,
                                      _p(h), _p(hu), _p(hv), _p(B), ctypes.byref(t))
    return h, hu, hv, t.value, st


def modular_stable_dt(p: _Grid, h, hu, hv):
    """(dt, status) of the modular solver's CFL guard (time_utils.hpp:14-38)."""
    out = ctypes.c_double(0.0)
    st = lib().swe_oracle_modular_stable_dt(ctypes.byref(p), _p(h), _p(hu), _p(hv),
                                            ctypes.byref(out))
    return out.value, st
