"""Seeded synthetic inputs for the shallow-water hot path.

The reference builds its inputs from TOML-selected initial conditions and
bathymetries (include/initial_condition/*.hpp, include/bathymetry/*.hpp).  The
workloads run here need a few it lacks (seeded multi-Gaussian bathymetry,
free-surface based dam break / lake at rest), so every input is generated once on
the host by this module and handed identically to the GPU path and to the CPU
oracle; RNG or libm differences therefore cannot break parity.

All arrays are full ghosted float64 ``(Nx + 4, Ny + 4)`` grids, row-major with
i = x (slow) and j = y (contiguous), ghosts included (nG = 2).  Cell centres are
``x = (i - nG + 0.5) * dx`` (include/core/grid.hpp:22-23), extended through the
ghost cells.
"""
from __future__ import annotations

import numpy as np

NG = 2


def centres(N: int, L: float = 1.0) -> np.ndarray:
    """Cell-centre coordinates of all N + 4 cells along one axis (ghosts included)."""
    d = L / N
    return (np.arange(N + 2 * NG, dtype=np.float64) - NG + 0.5) * d


def gauss_hump(Nx, Ny, Lx=1.0, Ly=1.0, h0=1.0, amp=0.1, x0=0.5, y0=0.5, two_sigma2=0.01):
    """h = h0 + amp * exp(-((x-x0)^2 + (y-y0)^2) / two_sigma2), hu = hv = 0, B = 0.

    With the defaults this is the 256^2 parity case: GaussInitial with peak 0.1 and
    2 sigma^2 = 0.01 (include/initial_condition/gauss_initial.hpp:13-28) over flat
    bathymetry b0 = 0.
    """
    x = centres(Nx, Lx)[:, None]
    y = centres(Ny, Ly)[None, :]
    h = h0 + amp * np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / two_sigma2)
    z = np.zeros_like(h)
    return np.ascontiguousarray(h), z.copy(), z.copy(), z.copy()


def fill_scalar_ghosts(a: np.ndarray, bc: str = "reflecting") -> np.ndarray:
    """Fills the ghost cells of a ghosted scalar field in place from the interior, as the
    reference does for the bathymetry after apply_bathymetry
    (apply_scalar_reflecting_bc, HPC_solver.hpp:373-404: mirrored rows for interior
    columns, then mirrored columns over all rows).  ``"transmissive"`` copies the
    nearest interior row / column instead (zero gradient)."""
    Nx, Ny = a.shape[0] - 2 * NG, a.shape[1] - 2 * NG
    refl = bc == "reflecting"
    for g in range(NG):
        src_lo = NG + g if refl else NG
        src_hi = NG + Nx - 1 - g if refl else NG + Nx - 1
        a[NG - 1 - g, NG:NG + Ny] = a[src_lo, NG:NG + Ny]
        a[NG + Nx + g, NG:NG + Ny] = a[src_hi, NG:NG + Ny]
    for g in range(NG):
        src_lo = NG + g if refl else NG
        src_hi = NG + Ny - 1 - g if refl else NG + Ny - 1
        a[:, NG - 1 - g] = a[:, src_lo]
        a[:, NG + Ny + g] = a[:, src_hi]
    return a


def gaussian_sum_bathymetry(Nx, Ny, n=16, seed=0, Lx=1.0, Ly=1.0, width=(0.02, 0.1),
                            amp=(-0.3, 0.3), rng=None, bc="reflecting"):
    """B = sum of n Gaussians with centres U[0,Lx]x[0,Ly], widths U[width], amplitudes U[amp].

    Each bump is a * exp(-((x-cx)^2 + (y-cy)^2) / (2 w^2)), evaluated at the interior
    cell centres; the ghosts are then filled for the wall type ``bc`` by
    :func:`fill_scalar_ghosts`, as the reference does for its GaussHill bathymetry
    (gaussian_hill.hpp:16-30 then HPC_solver.hpp:114), so a flat free surface is at rest
    up to the walls.  Separable, so it costs n outer products.
    Returns (B, params) with params an (n, 4) array of (cx, cy, w, a).
    """
    rng = np.random.default_rng(seed) if rng is None else rng
    cx = rng.uniform(0.0, Lx, n)
    cy = rng.uniform(0.0, Ly, n)
    w = rng.uniform(width[0], width[1], n)
    a = rng.uniform(amp[0], amp[1], n)
    x = centres(Nx, Lx)
    y = centres(Ny, Ly)
    B = np.zeros((Nx + 2 * NG, Ny + 2 * NG), dtype=np.float64)
    for m in range(n):
        gx = np.exp(-((x - cx[m]) ** 2) / (2.0 * w[m] ** 2))
        gy = np.exp(-((y - cy[m]) ** 2) / (2.0 * w[m] ** 2))
        B += a[m] * np.outer(gx, gy)
    fill_scalar_ghosts(B, bc)
    return B, np.stack([cx, cy, w, a], axis=1)


def dam_break(B, Lx=1.0, eta_left=1.5, eta_right=1.0, x_dam=0.4):
    """Free-surface dam break over B: eta = eta_left for x < x_dam else eta_right,
    h = max(0, eta - B), hu = hv = 0."""
    Nx = B.shape[0] - 2 * NG
    x = centres(Nx, Lx)[:, None]
    eta = np.where(x < x_dam, eta_left, eta_right)
    h = np.maximum(0.0, eta - B)
    z = np.zeros_like(h)
    return np.ascontiguousarray(h), z.copy(), z.copy()


def lake_at_rest(B, eta=1.0):
    """Still water with a flat free surface: h = max(0, eta - B), hu = hv = 0.

    (The reference's StillWater sets h = h0 instead, still_water.hpp:8-17, which is
    only at rest over flat bathymetry.)"""
    h = np.maximum(0.0, eta - B)
    z = np.zeros_like(h)
    return np.ascontiguousarray(h), z.copy(), z.copy()


def random_state(Nx, Ny, seed=0, h_range=(0.5, 1.5), q_scale=0.3, b_scale=0.2, dry_frac=0.0):
    """Rough random state for stress tests of every branch of the scheme.

    Optionally sets a fraction of cells nearly dry (h below the 1e-8 floor or
    exactly 0) so the dry-cell guards and positivity clamps are exercised."""
    rng = np.random.default_rng(seed)
    shape = (Nx + 2 * NG, Ny + 2 * NG)
    h = rng.uniform(h_range[0], h_range[1], shape)
    hu = rng.normal(0.0, q_scale, shape)
    hv = rng.normal(0.0, q_scale, shape)
    B = rng.normal(0.0, b_scale, shape)
    if dry_frac > 0:
        m = rng.random(shape) < dry_frac
        h[m] = rng.choice(np.array([0.0, 1e-9, 5e-9, 2e-8]), size=int(m.sum()))
        hu[m] *= 1e-8
        hv[m] *= 1e-8
    return h, hu, hv, B


def ensemble_instances(count=512, sizes=(128, 256, 512, 1024, 2048), seed=0):
    """The batched-ensemble workload: ``count`` square instances with side drawn uniformly
    from ``sizes``; each has its own Gaussian hump on eta = 1 (amplitude U[0.05, 0.3],
    centre U[0.2, 0.8]^2, width^2 U[0.002, 0.02]) over a bathymetry of 4 seeded
    Gaussians (centres U[0,1]^2, widths U[0.05, 0.15], amplitudes U[-0.2, 0.2]), u = v = 0,
    reflecting walls (bathymetry ghosts mirrored).

    Returns a list of (N, seed_q) pairs; :func:`ensemble_member` builds one member's
    arrays on demand so a 512-member ensemble never sits on the host all at once.
    """
    rng = np.random.default_rng(seed)
    sides = rng.choice(np.asarray(sizes), size=count)
    seeds = rng.integers(0, 2**31 - 1, size=count)
    return [(int(n), int(s)) for n, s in zip(sides, seeds)]


def ensemble_member(N, seed):
    """(h, hu, hv, B) of one ensemble member (see :func:`ensemble_instances`)."""
    rng = np.random.default_rng(seed)
    amp = rng.uniform(0.05, 0.3)
    cx, cy = rng.uniform(0.2, 0.8, size=2)
    w2 = rng.uniform(0.002, 0.02)
    B, _ = gaussian_sum_bathymetry(N, N, n=4, rng=rng, width=(0.05, 0.15), amp=(-0.2, 0.2),
                                   bc="reflecting")
    x = centres(N)[:, None]
    y = centres(N)[None, :]
    eta = 1.0 + amp * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / w2)
    h = np.maximum(0.0, eta - B)
    z = np.zeros_like(h)
    return np.ascontiguousarray(h), z.copy(), z.copy(), B
