"""Host-side mirror of the reference's optimised-backend interface, over the C ABI.

The reference's backends are C++ classes ``X(const SimulationConfig&)`` with
``run()`` (include/backend/serial/HPC/HPC_solver.hpp:88-200,
include/backend/cuda/cuda_solver.hpp:107-230).  :class:`Solver` wraps one
``swe_ctx`` (include/swe_gb300.h) with the same operations the reference performs
on its arrays (upload, rk3 steps, CFL dt, download); :meth:`Solver.run` mirrors
``FastHLLMUSCLBathySolver::run`` (fixed dt = end_time / time_steps, the one-off CFL
guard with the reference's message, and a snapshot every ``save_every`` steps).
Errors raise :class:`SweError` carrying the C status, as the reference throws
``std::runtime_error``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L

_BC = {"reflecting": L.SWE_BC_REFLECTING, "ReflectingWalls": L.SWE_BC_REFLECTING,
       "transmissive": L.SWE_BC_TRANSMISSIVE}
_PREC = {"fp64": L.SWE_PRECISION_FP64, "fp32_mixed": L.SWE_PRECISION_FP32_MIXED}


class SweError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ghosted(a, Nx, Ny, name):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != (Nx + 4, Ny + 4):
        raise ValueError(f"{name} must have shape {(Nx + 4, Ny + 4)} (ghosted), got {a.shape}")
    return a


class Solver:
    """One grid on one GPU.  Arrays are full ghosted ``(Nx+4, Ny+4)`` float64 grids."""

    def __init__(self, Nx: int, Ny: int, Lx: float = 1.0, Ly: float = 1.0,
                 g: float = 9.80665, cfl: float = 0.45, bc="reflecting",
                 precision="fp64", device: int = 0, x_halo=(False, False),
                 dx: float = 0.0, dy: float = 0.0, scheme: str = "fused",
                 reconstruction: str = "MUSCL", riemann: str = "HLL", bathymetry: bool = True):
        """``x_halo`` marks the low / high x sides whose ghost rows a neighbour slab
        supplies, ``dx``/``dy`` > 0 fix the cell sizes (see ``slabs.SlabGrid``).

        ``scheme="modular"`` runs the reference's SerialSolver arithmetic with the given
        ``reconstruction`` (PiecewiseConst, MUSCL), ``riemann`` (HLL, Rusanov, ROE) and
        ``bathymetry`` (False: the None instantiation, B unused); fixed dt only."""
        self._lib = L.lib()
        p = L.SweParams()
        self._lib.swe_params_default(ctypes.byref(p))
        p.Nx, p.Ny, p.Lx, p.Ly, p.g, p.cfl = Nx, Ny, Lx, Ly, g, cfl
        p.bc = _BC[bc] if isinstance(bc, str) else int(bc)
        p.precision = _PREC[precision] if isinstance(precision, str) else int(precision)
        p.device = device
        p.x_halo_lo, p.x_halo_hi = int(bool(x_halo[0])), int(bool(x_halo[1]))
        p.dx, p.dy = float(dx), float(dy)
        p.scheme = {"fused": L.SWE_SCHEME_FUSED, "modular": L.SWE_SCHEME_MODULAR}[scheme]
        p.reconstruction = L.RECONSTRUCTIONS[reconstruction]
        p.riemann = L.RIEMANN_SOLVERS[riemann]
        p.bathymetry = int(bool(bathymetry))
        self.params = p
        self.Nx, self.Ny = Nx, Ny
        self._ctx = ctypes.c_void_p()
        st = self._lib.swe_create(ctypes.byref(p), ctypes.byref(self._ctx))
        if st != L.SWE_OK:
            self._ctx = ctypes.c_void_p()
            raise SweError(st, "swe_create: " + self._lib.swe_status_string(st).decode())
        self.time = 0.0

    # -- plumbing -----------------------------------------------------------------
    def _check(self, st: int, what: str):
        if st != L.SWE_OK:
            msg = self._lib.swe_last_error(self._ctx).decode() if self._ctx else ""
            raise SweError(st, f"{what}: {self._lib.swe_status_string(st).decode()}: {msg}")

    def close(self):
        if self._ctx:
            self._lib.swe_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- the C ABI, one method each ------------------------------------------------
    def upload(self, h, hu, hv, B=None):
        h, hu, hv = (_ghosted(a, self.Nx, self.Ny, n) for a, n in ((h, "h"), (hu, "hu"), (hv, "hv")))
        Bp = None if B is None else _dp(_ghosted(B, self.Nx, self.Ny, "B"))
        self._keep = (h, hu, hv, B)
        self._check(self._lib.swe_upload(self._ctx, _dp(h), _dp(hu), _dp(hv), Bp), "swe_upload")

    def download(self, out=None):
        shape = (self.Nx + 4, self.Ny + 4)
        if out is None:
            out = tuple(np.empty(shape, dtype=np.float64) for _ in range(3))
        self._check(self._lib.swe_download(self._ctx, *(_dp(a) for a in out)), "swe_download")
        return out

    def step(self, n_steps: int = 1, dt: float | None = None) -> float:
        """Advances n_steps RK3 steps; dt None (or <= 0) = adaptive CFL dt.  Returns time."""
        t = ctypes.c_double(self.time)
        st = self._lib.swe_step(self._ctx, int(n_steps), float(dt or 0.0), ctypes.byref(t))
        self.time = t.value
        self._check(st, "swe_step")
        return self.time

    def step_host(self, h, hu, hv, B=None, out=None, n_steps: int = 1,
                  dt: float | None = None):
        """upload + step + download in one call (swe_step_host): the FP64 fused scheme
        overlaps the host transfers with the stage kernels.  ``out`` (three ghosted
        arrays, which may be the inputs) receives the state; returns ``out``."""
        h, hu, hv = (_ghosted(a, self.Nx, self.Ny, n) for a, n in ((h, "h"), (hu, "hu"), (hv, "hv")))
        Bp = None if B is None else _dp(_ghosted(B, self.Nx, self.Ny, "B"))
        shape = (self.Nx + 4, self.Ny + 4)
        if out is None:
            out = tuple(np.empty(shape, dtype=np.float64) for _ in range(3))
        for a in out:
            if a.shape != shape or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError(f"out arrays must be C-contiguous float64 {shape}")
        self._keep = (h, hu, hv, B)
        t = ctypes.c_double(self.time)
        st = self._lib.swe_step_host(self._ctx, _dp(h), _dp(hu), _dp(hv), Bp,
                                     *(_dp(a) for a in out), int(n_steps), float(dt or 0.0),
                                     ctypes.byref(t))
        self._check(st, "swe_step_host")
        self.time = t.value
        return out

    def stage(self, stage: int, dt: float):
        """One RK stage with fixed dt (swe_stage); stage s writes buffer s % 3."""
        self._check(self._lib.swe_stage(self._ctx, int(stage), float(dt)), "swe_stage")

    def halo_pack(self, buffer: int, side: int) -> np.ndarray:
        """The 2 interior rows next to x side ``side`` of ``buffer``: (3, 2, Ny + 4)."""
        rows = np.empty((3, 2, self.Ny + 4), dtype=np.float64)
        self._check(self._lib.swe_halo(self._ctx, int(buffer), int(side), 0, _dp(rows)),
                    "swe_halo")
        return rows

    def halo_unpack(self, buffer: int, side: int, rows: np.ndarray):
        """Writes (3, 2, Ny + 4) rows into the ghost rows of x side ``side``."""
        rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(3, 2, self.Ny + 4)
        self._check(self._lib.swe_halo(self._ctx, int(buffer), int(side), 1, _dp(rows)),
                    "swe_halo")

    def max_wave_speed(self) -> float:
        v = ctypes.c_double()
        self._check(self._lib.swe_max_wave_speed(self._ctx, ctypes.byref(v)), "swe_max_wave_speed")
        return v.value

    def stable_dt(self) -> float:
        v = ctypes.c_double()
        self._check(self._lib.swe_stable_dt(self._ctx, ctypes.byref(v)), "swe_stable_dt")
        return v.value

    def dt_log(self, n: int) -> np.ndarray:
        out = np.zeros(max(n, 1))
        w = ctypes.c_int()
        self._check(self._lib.swe_dt_log(self._ctx, _dp(out), n, ctypes.byref(w)), "swe_dt_log")
        return out[: w.value]

    def totals(self):
        """(mass, momentum_x, momentum_y) of the current state: compensated device sums
        of h, hu, hv over the interior times dx * dy."""
        v = [ctypes.c_double() for _ in range(3)]
        self._check(self._lib.swe_totals(self._ctx, *(ctypes.byref(x) for x in v)), "swe_totals")
        return tuple(x.value for x in v)

    def sanity(self):
        """On-device sanity reductions of the current state: mass (sum h dx dy), h_min,
        first_negative (row-major interior index i * Ny + j of the first h < 0, or -1, the
        cell the reference's Positivity check reports) and energy."""
        m, hmin, e = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        first = ctypes.c_longlong()
        self._check(self._lib.swe_sanity(self._ctx, ctypes.byref(m), ctypes.byref(hmin),
                                         ctypes.byref(first), ctypes.byref(e)), "swe_sanity")
        return {"mass": m.value, "h_min": hmin.value, "first_negative": first.value,
                "energy": e.value}

    def kernel_launches(self) -> int:
        return int(self._lib.swe_kernel_launches(self._ctx))

    def last_step_ms(self) -> float:
        """Device time (CUDA events on the library's stream) of the last step() call."""
        v = ctypes.c_double()
        self._check(self._lib.swe_last_step_ms(self._ctx, ctypes.byref(v)), "swe_last_step_ms")
        return v.value

    # -- FastHLLMUSCLBathySolver::run (HPC_solver.hpp:130-200) -----------------------
    def run(self, end_time: float, time_steps: int, save_every: int | None = None,
            on_snapshot=None, writer=None, bathymetry_name: str = ""):
        """Fixed-dt run as the reference: dt = end_time / time_steps, the CFL guard once
        before stepping, a snapshot (time, h, hu, hv) at t = 0 and every save_every
        steps and at the end, passed to ``on_snapshot`` and/or appended to ``writer``
        (an ``output.NetCDFWriter``; the first record carries the run metadata as
        cuda_solver.hpp:178-183 writes it, and records are written from the device while
        the run continues)."""
        dt = end_time / float(time_steps)
        dt_stable = self.stable_dt()
        if dt > dt_stable:
            raise SweError(L.SWE_ERR_CFL, f"Time step too large: dt = {dt:.6f}, but CFL "
                                          f"requires dt <= {dt_stable:.6f}")
        save_every = save_every or time_steps
        if on_snapshot:
            on_snapshot(0, self.time, *self.download())
        if writer is not None:
            bc = "Reflecting Walls" if self.params.bc == L.SWE_BC_REFLECTING else "Transmissive"
            writer.write_snapshot(self, self.time, dt, "GB300", "HLL", "MUSCL", "SSPRK3", bc,
                                  bathymetry_name)
        done = 0
        while done < time_steps:
            n = min(save_every - done % save_every, time_steps - done)
            self.step(n, dt)
            done += n
            if done % save_every == 0 or done == time_steps:
                if writer is not None:
                    writer.write_snapshot(self, self.time)
                if on_snapshot:
                    on_snapshot(done, self.time, *self.download())
        if writer is not None:
            writer.flush()
        return self.time
