"""FP32-mixed form on the GPU against the FP64 CPU oracle.

Stated tolerances: relative L1 error of h (sum |h - h_ref| / sum |h_ref| over the
interior) <= 1e-5 after the run; momentum errors are reported normwise.  A lake at
rest (all wet) must stay exactly at rest: eta bitwise constant, hu = hv = 0."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L1_H_TOL = 1e-5


def rel_l1(a, b):
    ai, bi = a[2:-2, 2:-2], b[2:-2, 2:-2]
    return float(np.abs(ai - bi).sum() / max(np.abs(bi).sum(), 1e-300))


def rel_linf(a, b):
    ai, bi = a[2:-2, 2:-2], b[2:-2, 2:-2]
    return float(np.abs(ai - bi).max() / max(np.abs(bi).max(), 1e-300))


def run_fp32(sw, h, hu, hv, B, Nx, Ny, steps, dt=None, bc=0, cfl=0.45, Lx=1.0, Ly=1.0):
    with sw.Solver(Nx, Ny, Lx, Ly, cfl=cfl, bc=bc, precision="fp32_mixed") as s:
        s.upload(h, hu, hv, B)
        s.step(steps, dt)
        return s.download(), s.time, s.dt_log(steps)


@pytest.mark.parametrize("bc", ["reflecting", "transmissive"])
def test_lake_at_rest_is_exact(gpu_lib, sw, problems, bc):
    B, _ = problems.gaussian_sum_bathymetry(128, 96, n=16, seed=4, amp=(-0.3, 0.4), bc=bc)
    h, hu, hv = problems.lake_at_rest(B, 1.0)
    assert h[2:-2, 2:-2].min() > 0.01
    (ho, huo, hvo), _, _ = run_fp32(sw, h, hu, hv, B, 128, 96, 300, dt=1e-3,
                                    bc=0 if bc == "reflecting" else 1)
    assert np.abs(huo).max() == 0.0 and np.abs(hvo).max() == 0.0
    # eta stays the FP32 image of 1.0 everywhere: h comes back as 1.0 - B32 in FP64
    want = 1.0 - B.astype(np.float32).astype(np.float64)
    assert np.array_equal(ho[2:-2, 2:-2], want[2:-2, 2:-2])


def test_gauss_hump_256_matches_fp64(gpu_lib, sw, port, problems):
    h, hu, hv, B = problems.gauss_hump(256, 256)
    p = port.grid(256, 256)
    dt = port.stable_dt(p, h, hu, hv)
    ref = port.run(p, h, hu, hv, B, 1000, dt)
    (ho, huo, hvo), t, _ = run_fp32(sw, h, hu, hv, B, 256, 256, 1000, dt=dt)
    assert rel_l1(ho, ref[0]) <= L1_H_TOL
    assert rel_linf(ho, ref[0]) <= 1e-4
    assert rel_linf(huo, ref[1]) <= 1e-3 and rel_linf(hvo, ref[2]) <= 1e-3
    # the FP32 form applies dt rounded to FP32 and accumulates that value in FP64
    t_want = 0.0
    for _ in range(1000):
        t_want += float(np.float32(dt))
    assert t == t_want


def test_dambreak_transmissive_matches_fp64(gpu_lib, sw, port, problems):
    N = 192
    B, _ = problems.gaussian_sum_bathymetry(N, N, n=16, seed=1, bc="transmissive")
    h, hu, hv = problems.dam_break(B)
    p = port.grid(N, N, bc=1)
    dt = 0.5 * port.stable_dt(p, h, hu, hv)
    ref = port.run(p, h, hu, hv, B, 150, dt)
    (ho, huo, hvo), _, _ = run_fp32(sw, h, hu, hv, B, N, N, 150, dt=dt, bc=1)
    assert rel_l1(ho, ref[0]) <= L1_H_TOL
    assert rel_l1(huo, ref[1]) <= 1e-3


def test_adaptive_dt_tracks_fp64(gpu_lib, sw, port, problems):
    N = 128
    B, _ = problems.gaussian_sum_bathymetry(N, N, n=16, seed=9, bc="transmissive")
    h, hu, hv = problems.dam_break(B)
    p = port.grid(N, N, bc=1)
    ref = port.run(p, h, hu, hv, B, 100, 0.0)
    (ho, _, _), t, dts = run_fp32(sw, h, hu, hv, B, N, N, 100, bc=1)
    assert np.abs(dts / ref[3] - 1.0).max() < 1e-5
    assert abs(t / ref[4] - 1.0) < 1e-5
    assert rel_l1(ho, ref[0]) <= L1_H_TOL


def test_mass_conserved_with_reflecting_walls(gpu_lib, sw, problems):
    h, hu, hv, B = problems.gauss_hump(200, 160)
    (ho, _, _), _, _ = run_fp32(sw, h, hu, hv, B, 200, 160, 400)
    m0 = h[2:-2, 2:-2].sum()
    m1 = ho[2:-2, 2:-2].sum()
    assert abs(m1 - m0) / m0 < 1e-6


def test_dry_cells_stay_nonnegative_and_finite(gpu_lib, sw, problems):
    B, _ = problems.gaussian_sum_bathymetry(96, 96, n=16, seed=5, amp=(-0.6, 1.6))
    h, hu, hv = problems.dam_break(B)
    assert (h[2:-2, 2:-2] == 0).any()
    (ho, huo, hvo), _, _ = run_fp32(sw, h, hu, hv, B, 96, 96, 200, cfl=0.3)
    assert np.isfinite(ho).all() and np.isfinite(huo).all() and np.isfinite(hvo).all()
    assert ho[2:-2, 2:-2].min() >= 0.0


def test_nonfinite_reports_status(gpu_lib, sw, problems):
    h, hu, hv, B = problems.random_state(16, 16, seed=1)
    hu[8, 8] = np.inf
    with sw.Solver(16, 16, precision="fp32_mixed") as s:
        s.upload(h, hu, hv, B)
        with pytest.raises(sw.SweError) as e:
            s.step(1, 1e-4)
        assert e.value.status == 3


def test_config2_16384_matches_fp64_gpu(gpu_lib, sw, problems):
    """The precision form at its own size (16384^2 dam break over the seeded 16-Gaussian
    bathymetry, transmissive walls) against an FP64 run of the same grid on the GPU,
    over a reduced step count: relative L1(h) within the stated budget."""
    n, steps = 16384, 20
    B, _ = problems.gaussian_sum_bathymetry(n, n, n=16, seed=2026, bc="transmissive")
    h, hu, hv = problems.dam_break(B)
    with sw.Solver(n, n, bc="transmissive") as s:
        s.upload(h, hu, hv, B)
        s.step(steps)
        ref = s.download()
    out, _, _ = run_fp32(sw, h, hu, hv, B, n, n, steps, bc=1)
    assert rel_l1(out[0], ref[0]) <= L1_H_TOL
