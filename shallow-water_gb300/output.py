"""NetCDF output over the C ABI: the reference's ``NetCDFWriter`` and
``SanityCheckNetCDFWriter`` (include/io/netCDF_writer.hpp:12-55,
include/io/sanity_checks_netdcdf_writer.hpp:5-41), with the same constructor
arguments, methods and file contents (dimensions, variables, attributes, values).

Files are written in the netCDF classic encoding by ``libswe_gb300.so`` itself
(CDF-2 for snapshots while every field is below 4 GiB, else CDF-5; CDF-5 for the
sanity records, whose ``step`` is uint64).  ``write_snapshot`` of a :class:`Solver`
packs the device state on the GPU and writes it from a background thread while the
solver keeps stepping; host arrays are written synchronously.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib as L
from .solver import Solver, SweError, _dp, _ghosted


def _b(s: str | None):
    return s.encode() if s else None


def _grid_of(grid):
    """(Nx, Ny, dx, dy) of a Solver, or of an (Nx, Ny, Lx, Ly) tuple (grid.hpp:19-20)."""
    if isinstance(grid, Solver):
        p = grid.params
        dx = p.dx if p.dx > 0 else p.Lx / p.Nx
        dy = p.dy if p.dy > 0 else p.Ly / p.Ny
        return grid.Nx, grid.Ny, dx, dy
    Nx, Ny, Lx, Ly = grid
    return int(Nx), int(Ny), float(Lx) / int(Nx), float(Ly) / int(Ny)


class NetCDFWriter:
    """Snapshot file: ``time`` (unlimited), ``x``, ``y``; ``h``, ``hu``, ``hv`` per record,
    ``B`` once, cell-centre coordinates, units and run metadata as attributes."""

    def __init__(self, path: str, grid, spatial_unit_x: str = "", spatial_unit_y: str = "",
                 spatial_unit_h: str = "", time_unit: str = "", save_every: int = 1,
                 format: int = 0):
        self._lib = L.lib()
        self.Nx, self.Ny, self.dx, self.dy = _grid_of(grid)
        p = L.SnapshotParams()
        p.Nx, p.Ny, p.dx, p.dy = self.Nx, self.Ny, self.dx, self.dy
        p.unit_x, p.unit_y = _b(spatial_unit_x), _b(spatial_unit_y)
        p.unit_h, p.unit_time = _b(spatial_unit_h), _b(time_unit)
        p.save_every, p.format = int(save_every), int(format)
        self._s = ctypes.c_void_p()
        st = self._lib.swe_snapshot_open(str(path).encode(), ctypes.byref(p), ctypes.byref(self._s))
        if st != L.SWE_OK:
            self._s = ctypes.c_void_p()
            raise SweError(st, f"swe_snapshot_open({path}): "
                               + self._lib.swe_status_string(st).decode())
        self.path = str(path)

    def _check(self, st: int, what: str):
        if st != L.SWE_OK:
            msg = self._lib.swe_snapshot_last_error(self._s).decode() if self._s else ""
            raise SweError(st, f"{what}: {self._lib.swe_status_string(st).decode()}: {msg}")

    def write_bathymetry(self, B: np.ndarray):
        B = _ghosted(B, self.Nx, self.Ny, "B")
        self._check(self._lib.swe_snapshot_bathymetry(self._s, _dp(B)), "write_bathymetry")

    def write_snapshot(self, U, time: float, dt: float = math.nan, backend: str = "",
                       riemann_solver: str = "", reconstruction: str = "",
                       time_integrator: str = "", boundary_condition: str = "",
                       bathymetry: str = ""):
        """U: a :class:`Solver` (its current device state, written asynchronously) or
        ghosted host arrays ``(h, hu, hv)`` (written before returning)."""
        self._check(self._lib.swe_snapshot_metadata(
            self._s, float(dt), _b(backend), _b(riemann_solver), _b(reconstruction),
            _b(time_integrator), _b(boundary_condition), _b(bathymetry)), "write_snapshot")
        if isinstance(U, Solver):
            self._check(self._lib.swe_snapshot_write(self._s, U._ctx, float(time)),
                        "write_snapshot")
            return
        h, hu, hv = (_ghosted(a, self.Nx, self.Ny, n) for a, n in zip(U, ("h", "hu", "hv")))
        self._check(self._lib.swe_snapshot_write_host(self._s, float(time), _dp(h), _dp(hu),
                                                      _dp(hv)), "write_snapshot")

    @property
    def records(self) -> int:
        return int(self._lib.swe_snapshot_records(self._s))

    def stats(self):
        """(device-to-host seconds, file-write seconds, bytes) of the device records."""
        c, w, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        self._check(self._lib.swe_snapshot_stats(self._s, ctypes.byref(c), ctypes.byref(w),
                                                 ctypes.byref(n)), "stats")
        return c.value, w.value, n.value

    def flush(self):
        self._check(self._lib.swe_snapshot_flush(self._s), "flush")

    def close(self):
        if self._s:
            st = self._lib.swe_snapshot_close(self._s)
            msg = self._lib.swe_snapshot_last_error(self._s).decode()
            self._lib.swe_snapshot_destroy(self._s)
            self._s = ctypes.c_void_p()
            if st != L.SWE_OK:
                raise SweError(st, f"close: {self._lib.swe_status_string(st).decode()}: {msg}")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            if self._s:
                self._lib.swe_snapshot_destroy(self._s)
                self._s = ctypes.c_void_p()
        except Exception:
            pass


class SanityCheckNetCDFWriter:
    """Sanity records ``step``, ``time``, ``mass_rel_err``, ``h_min`` per record
    (sanity_checks_netcdf_writer.cpp:25-71)."""

    def __init__(self, path: str, time_unit: str, h_unit: str, save_every: int, dt: float,
                 backend_name: str, riemann_solver: str, reconstruction: str,
                 time_integrator: str, boundary_condition: str, bathymetry: str):
        self._lib = L.lib()
        self._l = ctypes.c_void_p()
        st = self._lib.swe_sanity_log_open(
            str(path).encode(), _b(time_unit), _b(h_unit), int(save_every), float(dt),
            _b(backend_name), _b(riemann_solver), _b(reconstruction), _b(time_integrator),
            _b(boundary_condition), _b(bathymetry), ctypes.byref(self._l))
        if st != L.SWE_OK:
            self._l = ctypes.c_void_p()
            raise SweError(st, f"swe_sanity_log_open({path}): "
                               + self._lib.swe_status_string(st).decode())
        self.path = str(path)

    def write(self, step: int, time: float, rel_err: float, h_min: float):
        st = self._lib.swe_sanity_log_write(self._l, int(step), float(time), float(rel_err),
                                            float(h_min))
        if st != L.SWE_OK:
            raise SweError(st, "write: " + self._lib.swe_sanity_log_last_error(self._l).decode())

    def close(self):
        if self._l:
            st = self._lib.swe_sanity_log_close(self._l)
            msg = self._lib.swe_sanity_log_last_error(self._l).decode()
            self._lib.swe_sanity_log_destroy(self._l)
            self._l = ctypes.c_void_p()
            if st != L.SWE_OK:
                raise SweError(st, "close: " + msg)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            if self._l:
                self._lib.swe_sanity_log_destroy(self._l)
                self._l = ctypes.c_void_p()
        except Exception:
            pass
