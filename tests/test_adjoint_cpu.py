"""CPU checks of the discrete adjoint's building blocks, no GPU needed:
the interface VJP against central differences and against its textbook derivation
(tests/cpp/adjoint_face_textbook.h), and the assembled adjoint (ghost folding,
divergence, RK3 stages, positivity masks) of tests/cpp/adjoint_ref.cpp against central
differences of the same forward, along random directions."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.skipif(not shutil.which("g++"), reason="g++ not available")


def test_interface_vjp_matches_finite_differences(tmp_path):
    exe = tmp_path / "adj_face"
    subprocess.run(["g++", "-std=c++17", "-O2", "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "adjoint_face_check.cpp")], check=True)
    r = subprocess.run([str(exe), "20000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    assert " 0 bad" in r.stdout
    # and the per-side-sum derivation agrees with the textbook one to rounding
    assert " 0 differ" in r.stdout


def smooth_case(problems, Nx, Ny, bc, seed):
    rng = np.random.default_rng(seed)
    bcs = "reflecting" if bc == 0 else "transmissive"
    B, _ = problems.gaussian_sum_bathymetry(Nx, Ny, n=3, rng=rng, width=(0.15, 0.3),
                                            amp=(-0.1, 0.1), bc=bcs)
    x = problems.centres(Nx)[:, None]
    y = problems.centres(Ny)[None, :]
    eta = 1.0 + 0.05 * np.exp(-((x - 0.4) ** 2 + (y - 0.6) ** 2) / 0.05)
    # noise breaks exact symmetries: a zero slope is a kink of minmod, where central
    # differences average two one-sided derivatives
    eta = eta + 1e-3 * rng.standard_normal(eta.shape)
    # far from the bumps B is ~1e-30 and max(b-, b+) would flip under the perturbation
    B = B + 1e-3 * rng.standard_normal(B.shape)
    problems.fill_scalar_ghosts(B, bcs)
    h = eta - B
    hu = 0.02 * np.sin(3 * x + y) + 1e-3 * rng.standard_normal(eta.shape)
    hv = 0.015 * np.cos(2 * y - x) + 1e-3 * rng.standard_normal(eta.shape)
    return h, hu, hv, B, rng


def smooth_direction(problems, Nx, Ny, rng):
    """A random smooth perturbation (sum of 4 random Gaussian bumps, interior only).
    Per-cell white noise would move neighbouring differences by ~eps and cross the
    kinks of minmod and max(b-, b+); smooth directions move them by ~eps * dx."""
    d, _ = problems.gaussian_sum_bathymetry(Nx, Ny, n=4, rng=rng, width=(0.1, 0.3),
                                            amp=(-1.0, 1.0))
    d[:2, :] = d[-2:, :] = 0.0
    d[:, :2] = d[:, -2:] = 0.0
    return d


@pytest.mark.parametrize("bc", [0, 1], ids=["reflecting", "transmissive"])
def test_full_adjoint_matches_finite_differences(problems, bc):
    import adjref
    Nx, Ny, steps, dt = 12, 10, 8, 2e-3
    h, hu, hv, B, rng = smooth_case(problems, Nx, Ny, bc, seed=5 + bc)
    ng = 5
    gi, gj = rng.integers(0, Nx, ng), rng.integers(0, Ny, ng)
    obs = 1.0 + 0.01 * rng.standard_normal((steps, ng))
    J, gh, ghu, ghv, gB = adjref.run(Nx, Ny, h, hu, hv, B, steps, dt, gi, gj, obs, bc=bc)
    bcs = "reflecting" if bc == 0 else "transmissive"
    eps = 1e-7  # see tests/test_adjoint_gpu.py on kinks of the scheme
    for trial in range(4):
        dirs = [smooth_direction(problems, Nx, Ny, rng) for _ in range(4)]
        dB = dirs[3].copy()
        problems.fill_scalar_ghosts(dB, bcs)

        def J_at(s):
            return adjref.run(Nx, Ny, h + s * dirs[0], hu + s * dirs[1], hv + s * dirs[2],
                              B + s * dB, steps, dt, gi, gj, obs, grads=False, bc=bc)

        fd = (J_at(eps) - J_at(-eps)) / (2 * eps)
        ad = sum(float((g[2:-2, 2:-2] * d[2:-2, 2:-2]).sum()) for g, d in
                 zip((gh, ghu, ghv, gB), dirs))
        assert abs(fd - ad) <= 1e-6 * max(abs(fd), 1e-3), (trial, fd, ad)
