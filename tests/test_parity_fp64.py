"""FP64 drop-in on the GPU, through the C ABI, against the CPU oracle: bitwise equal
fields, dt sequences and times (max relative error 0 <= 1e-12)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import bitwise_equal, max_rel_err

pytestmark = pytest.mark.gpu


def run_both(sw, port, h, hu, hv, B, Nx, Ny, steps, dt=0.0, Lx=1.0, Ly=1.0, cfl=0.45, bc=0,
             g=9.80665, chunks=1):
    p = port.grid(Nx, Ny, Lx, Ly, g=g, cfl=cfl, bc=bc)
    ref = port.run(p, h, hu, hv, B, steps, dt)
    with sw.Solver(Nx, Ny, Lx, Ly, g=g, cfl=cfl, bc=bc) as s:
        s.upload(h, hu, hv, B)
        dts = []
        per = steps // chunks
        for c in range(chunks):
            n = per if c < chunks - 1 else steps - per * (chunks - 1)
            s.step(n, dt if dt > 0 else None)
            dts.append(s.dt_log(n))
        out = s.download()
        return ref, out, np.concatenate(dts), s.time, s


def assert_bitwise(ref, out, dts, t):
    assert ref[5] == 0
    for k, name in enumerate(("h", "hu", "hv")):
        err = max_rel_err(out[k], ref[k])
        assert err <= 1e-12, (name, err)
        assert bitwise_equal(out[k], ref[k]), (name, err)
    assert bitwise_equal(dts, ref[3])
    assert t == ref[4]


@pytest.mark.parametrize("g", [9.80665, 9.81])
def test_config0_small_gauss_hump(gpu_lib, sw, port, problems, g):
    h, hu, hv, B = problems.gauss_hump(64, 64)
    p = port.grid(64, 64, g=g)
    dt = port.stable_dt(p, h, hu, hv)
    ref, out, dts, t, _ = run_both(sw, port, h, hu, hv, B, 64, 64, 200, dt=dt, g=g)
    assert_bitwise(ref, out, dts, t)


def test_config0_full_256_1000_steps(gpu_lib, sw, port, problems):
    """The 256^2, 1000-step parity case (CFL 0.45 fixed dt)."""
    h, hu, hv, B = problems.gauss_hump(256, 256)
    dt = port.stable_dt(port.grid(256, 256), h, hu, hv)
    ref, out, dts, t, _ = run_both(sw, port, h, hu, hv, B, 256, 256, 1000, dt=dt, chunks=4)
    assert_bitwise(ref, out, dts, t)


@pytest.mark.parametrize("bc", [0, 1], ids=["reflecting", "transmissive"])
@pytest.mark.parametrize("shape", [(37, 29), (2, 2), (3, 130), (130, 3), (64, 96)])
def test_random_states_adaptive(gpu_lib, sw, port, problems, bc, shape):
    Nx, Ny = shape
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=Nx * 1000 + Ny, q_scale=0.1, b_scale=0.05)
    ref, out, dts, t, _ = run_both(sw, port, h, hu, hv, B, Nx, Ny, 15, cfl=0.3, bc=bc,
                                   Lx=1.0, Ly=1.7)
    assert_bitwise(ref, out, dts, t)


def test_dry_cells_and_positivity(gpu_lib, sw, port, problems):
    h, hu, hv, B = problems.random_state(48, 40, seed=9, q_scale=0.1, b_scale=0.05, dry_frac=0.1)
    ref, out, dts, t, _ = run_both(sw, port, h, hu, hv, B, 48, 40, 20, cfl=0.2)
    assert_bitwise(ref, out, dts, t)


@pytest.mark.parametrize("bc", [0, 1], ids=["reflecting", "transmissive"])
def test_wave_speed_of_dry_and_near_dry_cells(gpu_lib, sw, port, problems, bc):
    """The per-cell wave speed's branches, bitwise through the dt sequence: dry cells
    (h <= 1e-8, including exactly 1e-8 and 0) carrying large momenta, whose velocity the
    scheme takes as zero (a speed from |hu| / h there would be ~1e8 and set dt), beside
    near-dry wet cells (h just above 1e-8) whose large velocity sets the max speed, and
    ordinary wet cells."""
    Nx, Ny = 72, 56
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=41 + bc, q_scale=0.2, b_scale=0.05)
    rng = np.random.default_rng(43 + bc)
    dry = rng.random(h.shape) < 0.08
    h[dry] = rng.choice(np.array([0.0, 3e-9, 1e-8]), size=int(dry.sum()))
    hu[dry] = rng.choice(np.array([-2.0, 1.0, 3.0]), size=int(dry.sum()))
    hv[dry] = rng.choice(np.array([-1.5, 0.5, 2.5]), size=int(dry.sum()))
    fast = ~dry & (rng.random(h.shape) < 0.01)
    h[fast] = 2.5e-8
    hu[fast] = rng.choice(np.array([-1e-6, 5e-7]), size=int(fast.sum()))  # |u| up to 40
    hv[fast] = 3e-7
    ref, out, dts, t, _ = run_both(sw, port, h, hu, hv, B, Nx, Ny, 12, cfl=0.3, bc=bc, chunks=3)
    assert_bitwise(ref, out, dts, t)
    # the first dt is set by a near-dry cell's speed (|u| = 40), neither by the wet cells
    # (about 4.5) nor by a dry cell's momentum over its depth (up to 1e9)
    dx = 1.0 / Nx
    assert 0.3 * dx / 100.0 < dts[0] < 0.3 * dx / 20.0, dts[0]


def test_dambreak_transmissive(gpu_lib, sw, port, problems):
    B, _ = problems.gaussian_sum_bathymetry(200, 136, n=16, seed=2, bc="transmissive")
    h, hu, hv = problems.dam_break(B)
    ref, out, dts, t, _ = run_both(sw, port, h, hu, hv, B, 200, 136, 60, bc=1, chunks=3)
    assert_bitwise(ref, out, dts, t)


@pytest.mark.parametrize("bc", ["reflecting", "transmissive"])
def test_lake_at_rest_all_wet_is_exact(gpu_lib, sw, port, problems, bc):
    """Submerged bumps, eta = 1: momentum stays at rounding level (reference behaviour)."""
    B, _ = problems.gaussian_sum_bathymetry(96, 96, n=8, seed=4, amp=(-0.3, 0.5), bc=bc)
    h, hu, hv = problems.lake_at_rest(B, 1.0)
    assert h[2:-2, 2:-2].min() > 0.1
    ref, out, dts, t, _ = run_both(sw, port, h, hu, hv, B, 96, 96, 100, dt=1e-3,
                                   bc=0 if bc == "reflecting" else 1)
    assert_bitwise(ref, out, dts, t)
    assert np.abs(out[1]).max() < 1e-13 and np.abs(out[2]).max() < 1e-13


def test_golden_fixtures_on_gpu(gpu_lib, sw):
    from test_golden import SMALL, load_case
    for name in SMALL:
        meta, a = load_case(name)
        with sw.Solver(meta["Nx"], meta["Ny"], meta["Lx"], meta["Ly"], cfl=meta["cfl"],
                       bc=meta["bc"]) as s:
            s.upload(a["h"], a["hu"], a["hv"], a["B"])
            s.step(meta["steps"], meta["dt_fixed"] or None)
            out = s.download()
            assert bitwise_equal(out[0], a["h_out"]), name
            assert bitwise_equal(out[1], a["hu_out"]), name
            assert bitwise_equal(out[2], a["hv_out"]), name
            assert bitwise_equal(s.dt_log(meta["steps"]), a["dts"]), name
            assert s.time == meta["t_end"], name


def test_stable_dt_and_speed(gpu_lib, sw, port, problems):
    h, hu, hv, B = problems.random_state(50, 70, seed=1)
    p = port.grid(50, 70, 2.0, 1.0)
    with sw.Solver(50, 70, 2.0, 1.0) as s:
        s.upload(h, hu, hv, B)
        assert s.max_wave_speed() == port.max_wave_speed(p, h, hu, hv)
        assert s.stable_dt() == port.stable_dt(p, h, hu, hv)


def test_nonfinite_reports_status(gpu_lib, sw, problems):
    h, hu, hv, B = problems.random_state(16, 16, seed=1)
    h[8, 8] = np.nan
    with sw.Solver(16, 16) as s:
        s.upload(h, hu, hv, B)
        with pytest.raises(sw.SweError) as e:
            s.step(1, 1e-4)
        assert e.value.status == 3
        # the context stays usable after the error
        h2, hu2, hv2, B2 = problems.random_state(16, 16, seed=2)
        s.upload(h2, hu2, hv2, B2)
        s.step(2, None)


def test_cfl_guard_in_run(gpu_lib, sw, problems):
    h, hu, hv, B = problems.gauss_hump(32, 32)
    with sw.Solver(32, 32) as s:
        s.upload(h, hu, hv, B)
        with pytest.raises(sw.SweError) as e:
            s.run(end_time=1.0, time_steps=10)
        assert e.value.status == 4 and "Time step too large" in str(e.value)


def test_run_snapshots_match_oracle(gpu_lib, sw, port, problems):
    h, hu, hv, B = problems.gauss_hump(40, 40)
    p = port.grid(40, 40)
    dt = port.stable_dt(p, h, hu, hv)
    snaps = []
    with sw.Solver(40, 40) as s:
        s.upload(h, hu, hv, B)
        s.run(end_time=dt * 30, time_steps=30, save_every=10,
              on_snapshot=lambda n, t, a, b, c: snaps.append((n, a.copy())))
    assert [n for n, _ in snaps] == [0, 10, 20, 30]
    ref = port.run(p, h, hu, hv, B, 30, (dt * 30) / 30.0)
    assert bitwise_equal(snaps[-1][1], ref[0])


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_totals_are_compensated_sums(gpu_lib, sw, problems, precision):
    """swe_totals is within its error bound of the exactly rounded sum (math.fsum) of the
    downloaded state: plain sums of 8-cell chunks (7 roundings each) merged with
    error-free TwoSum, so |error| <= about 9 eps times the sum of magnitudes."""
    import math
    h, hu, hv, B = problems.random_state(300, 257, seed=3, q_scale=0.2, b_scale=0.05)
    with sw.Solver(300, 257, 1.0, 1.3, precision=precision) as s:
        s.upload(h, hu, hv, B)
        s.step(3)
        mass, mx, my = s.totals()
        out = s.download()
    dxdy = (1.0 / 300) * (1.3 / 257)
    for got, a in zip((mass, mx, my), out):
        want = math.fsum(a[2:-2, 2:-2].ravel()) * dxdy
        assert abs(got - want) <= 1e-15 * max(abs(want), math.fsum(np.abs(a[2:-2, 2:-2]).ravel()) * dxdy)


def test_config1_8192_dambreak_bitwise_two_steps(gpu_lib, sw, port, problems):
    """The headline workload at its own size (8192^2 dam break over 16 seeded Gaussians,
    transmissive walls, adaptive dt) against the CPU oracle over a reduced step count."""
    n = 8192
    B, _ = problems.gaussian_sum_bathymetry(n, n, n=16, seed=2026, bc="transmissive")
    h, hu, hv = problems.dam_break(B)
    ref, out, dts, t, _ = run_both(sw, port, h, hu, hv, B, n, n, 2, bc=1)
    assert_bitwise(ref, out, dts, t)


def test_config1_8192_lake_at_rest_stays_at_rest(gpu_lib, sw, problems):
    """The lake-at-rest run of the 8192^2 configuration (eta = 1 over the same
    bathymetry, u = v = 0): velocities stay at rounding level where the lake is wet."""
    n = 8192
    B, _ = problems.gaussian_sum_bathymetry(n, n, n=16, seed=2026, bc="transmissive")
    h, hu, hv = problems.lake_at_rest(B)
    with sw.Solver(n, n, bc="transmissive") as s:
        s.upload(h, hu, hv, B)
        s.step(20)
        oh, ohu, ohv = s.download()
    wet = h[2:-2, 2:-2] > 1e-3
    assert wet.mean() > 0.5
    assert np.abs(ohu[2:-2, 2:-2][wet]).max() < 1e-12
    assert np.abs(ohv[2:-2, 2:-2][wet]).max() < 1e-12
