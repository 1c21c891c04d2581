"""Gradients of a gauge-misfit objective through the discrete adjoint (swe_adjoint_gauge).

J = sum over steps n = 1..N and gauges q of (h^n at gauge q - h_obs[n-1, q])^2, for N
fixed-dt SSP-RK3 steps, through the FP64 or the FP32-mixed scheme (the solver's).  :func:`gauge_misfit_gradient` returns J and its gradients with
respect to the initial state and the bathymetry; :class:`GaugeMisfit` wraps it as a
``torch.autograd.Function`` of the initial free surface eta0 and the bathymetry B
(interior arrays; h0 = eta0 - B, hu0 = hv0 = 0).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from . import problems
from .solver import Solver, _dp


def gauge_misfit_gradient(solver: Solver, steps: int, dt: float, gauges, h_obs,
                          snapshots: int | None = None):
    """Runs the adjoint from the solver's current state (left unchanged).

    ``gauges`` is a sequence of (i, j) interior cells, ``h_obs`` a (steps, n_gauges)
    array.  ``snapshots`` stored states drive the binomial checkpoint schedule (default
    about sqrt(steps)); ``snapshots="tape"`` keeps every state and every step's stage
    states instead (no recomputation, about 75 bytes per cell and step);
    ``snapshots="segments"`` stores the state every sqrt(steps) steps and recomputes each
    segment once with its stage states kept (every step but the last segment's advanced
    twice).  Returns a dict with J, grad_h, grad_hu, grad_hv, grad_B (ghosted
    arrays, zero ghosts; grad_B holds the initial state fixed) and ms (device time)."""
    g = np.asarray(gauges, dtype=np.int32).reshape(-1, 2)
    gi = np.ascontiguousarray(g[:, 0])
    gj = np.ascontiguousarray(g[:, 1])
    obs = np.ascontiguousarray(h_obs, dtype=np.float64).reshape(steps, len(gi))
    if snapshots is None:
        snapshots = max(1, int(round(np.sqrt(steps))))
    elif snapshots == "tape":
        snapshots = L.ADJ_TAPE_ALL
    elif snapshots == "segments":
        snapshots = L.ADJ_SEGMENTS
    shape = (solver.Nx + 4, solver.Ny + 4)
    out = [np.zeros(shape) for _ in range(4)]
    J = ctypes.c_double()
    ms = ctypes.c_double()
    ip = ctypes.POINTER(ctypes.c_int)
    st = solver._lib.swe_adjoint_gauge(solver._ctx, int(steps), float(dt), len(gi),
                                       gi.ctypes.data_as(ip), gj.ctypes.data_as(ip), _dp(obs),
                                       int(snapshots), ctypes.byref(J), *(_dp(a) for a in out),
                                       ctypes.byref(ms))
    solver._check(st, "swe_adjoint_gauge")
    return {"J": J.value, "grad_h": out[0], "grad_hu": out[1], "grad_hv": out[2],
            "grad_B": out[3], "ms": ms.value}


def gauge_misfit(solver: Solver, steps: int, dt: float, gauges, h_obs):
    """J alone, from the solver's current state (left unchanged): one forward sweep
    through the same stage kernels and gauge sum as :func:`gauge_misfit_gradient`, so the
    value is bitwise that call's J.  Returns (J, device ms)."""
    g = np.asarray(gauges, dtype=np.int32).reshape(-1, 2)
    gi = np.ascontiguousarray(g[:, 0])
    gj = np.ascontiguousarray(g[:, 1])
    obs = np.ascontiguousarray(h_obs, dtype=np.float64).reshape(steps, len(gi))
    J, ms = ctypes.c_double(), ctypes.c_double()
    ip = ctypes.POINTER(ctypes.c_int)
    st = solver._lib.swe_adjoint_gauge(solver._ctx, int(steps), float(dt), len(gi),
                                       gi.ctypes.data_as(ip), gj.ctypes.data_as(ip), _dp(obs),
                                       0, ctypes.byref(J), None, None, None, None,
                                       ctypes.byref(ms))
    solver._check(st, "swe_adjoint_gauge")
    return J.value, ms.value


def gauge_series(solver: Solver, steps: int, dt: float, gauges) -> np.ndarray:
    """h at the gauge cells after each of ``steps`` fixed-dt steps from the solver's
    current state, which the run advances: the (steps, n_gauges) observations of a
    forward run, as the misfit compares them."""
    g = np.asarray(gauges, dtype=np.int64).reshape(-1, 2)
    out = np.empty((steps, len(g)))
    for k in range(steps):
        solver.step(1, dt)
        h = solver.download()[0]
        out[k] = h[g[:, 0] + 2, g[:, 1] + 2]
    return out


def ghosted_state(eta0, B, bc="reflecting"):
    """Ghosted (h, hu, hv, B) from interior eta0 and B: B's ghosts follow the wall rule,
    h0 = max(0, eta0 - B), hu0 = hv0 = 0."""
    Nx, Ny = eta0.shape
    Bg = np.zeros((Nx + 4, Ny + 4))
    Bg[2:-2, 2:-2] = B
    problems.fill_scalar_ghosts(Bg, bc)
    h = np.zeros_like(Bg)
    h[2:-2, 2:-2] = np.maximum(0.0, eta0 - B)
    return h, np.zeros_like(h), np.zeros_like(h), Bg


try:
    import torch

    class GaugeMisfit(torch.autograd.Function):
        """J(eta0, B) with gradients from the GPU discrete adjoint.

        ``GaugeMisfit.apply(eta0, B, steps, dt, gauges, h_obs, Lx, Ly, g, bc, snapshots,
        precision)``; eta0 and B are float64 (Nx, Ny) tensors; precision "fp32_mixed" runs
        the FP32 forward and adjoint.  Backward returns
        dJ/deta0 = dJ/dh0 and dJ/dB = (dJ/dB at fixed h0) - dJ/dh0 (h0 = eta0 - B, wet)."""

        @staticmethod
        def forward(ctx, eta0, B, steps, dt, gauges, h_obs, Lx=1.0, Ly=1.0, g=9.80665,
                    bc="reflecting", snapshots=None, precision="fp64"):
            e = eta0.detach().cpu().double().numpy()
            b = B.detach().cpu().double().numpy()
            h, hu, hv, Bg = ghosted_state(e, b, bc)
            Nx, Ny = e.shape
            with Solver(Nx, Ny, Lx, Ly, g=g, bc=bc, precision=precision) as s:
                s.upload(h, hu, hv, Bg)
                r = gauge_misfit_gradient(s, steps, dt, gauges, np.asarray(h_obs), snapshots)
            wet = (e - b) > 0
            g_eta = np.where(wet, r["grad_h"][2:-2, 2:-2], 0.0)
            g_B = r["grad_B"][2:-2, 2:-2] - g_eta
            ctx.save_for_backward(torch.from_numpy(g_eta).to(eta0.device),
                                  torch.from_numpy(g_B).to(B.device))
            return torch.tensor(r["J"], dtype=torch.float64, device=eta0.device)

        @staticmethod
        def backward(ctx, gJ):
            g_eta, g_B = ctx.saved_tensors
            return (gJ * g_eta, gJ * g_B) + (None,) * 10
except ImportError:  # pragma: no cover - torch is optional for the C ABI users
    GaugeMisfit = None
