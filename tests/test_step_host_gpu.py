"""swe_step_host (upload + step + download in one call, transfers overlapped with the
stage kernels by bands of rows) against the three separate calls and the oracle:
bitwise equal fields, ghosts, dt sequences and times, on grids of one to several
bands, ragged last tiles, both walls, adaptive and fixed dt, in-place outputs."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import bitwise_equal

pytestmark = pytest.mark.gpu


def sequence(sw, Nx, Ny, h, hu, hv, B, n, dt, **kw):
    with sw.Solver(Nx, Ny, **kw) as s:
        s.upload(h, hu, hv, B)
        s.step(n, dt)
        return s.download(), s.time, s.dt_log(n)


def same(a, b):
    return all(bitwise_equal(x, y) for x, y in zip(a, b))


# (Nx, Ny): one band; 65 tile rows (two bands); 129 tile rows with a last tile row of
# one grid row (three bands); wide rows, several bands; 257 tile rows, where the first
# and the last band are quarter bands (16 tile rows) around four full ones
SHAPES = [(20, 14), (520, 40), (1025, 70), (1037, 203), (2049, 36)]


@pytest.mark.parametrize("bc", ["reflecting", "transmissive"])
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: f"{s[0]}x{s[1]}")
def test_matches_separate_calls(gpu_lib, sw, problems, bc, shape):
    Nx, Ny = shape
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=Nx + Ny, q_scale=0.1, b_scale=0.05,
                                         dry_frac=0.02)
    for n, dt in ((1, None), (3, None), (2, 1e-5)):
        want, t, dts = sequence(sw, Nx, Ny, h, hu, hv, B, n, dt, bc=bc, cfl=0.3)
        with sw.Solver(Nx, Ny, bc=bc, cfl=0.3) as s:
            got = s.step_host(h, hu, hv, B, n_steps=n, dt=dt)
            assert same(got, want), (n, dt)
            assert s.time == t
            assert bitwise_equal(s.dt_log(n), dts)


def test_matches_oracle_and_chains(gpu_lib, sw, port, problems):
    """Two calls in a row, the second on the first's output with B omitted, equal the
    oracle's run of all the steps."""
    Nx, Ny = 300, 97
    B, _ = problems.gaussian_sum_bathymetry(Nx, Ny, n=8, seed=4, bc="transmissive")
    h, hu, hv = problems.dam_break(B)
    ref = port.run(port.grid(Nx, Ny, bc=1), h, hu, hv, B, 7, 0.0)
    assert ref[5] == 0
    with sw.Solver(Nx, Ny, bc="transmissive") as s:
        out = s.step_host(h, hu, hv, B, n_steps=4)
        out = s.step_host(*out, n_steps=3)
        dts = s.dt_log(3)
    for k in range(3):
        assert bitwise_equal(out[k], ref[k])
    assert bitwise_equal(dts, ref[3][4:])


def test_in_place_pinned(gpu_lib, sw, problems):
    """Page-locked host arrays (the overlapped path), outputs written over the inputs."""
    Nx, Ny = 1100, 64
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=5, q_scale=0.1, b_scale=0.05)
    want, t, _ = sequence(sw, Nx, Ny, h, hu, hv, B, 2, None)
    pin = [torch.empty((Nx + 4, Ny + 4), dtype=torch.float64, pin_memory=True).numpy()
           for _ in range(4)]
    for dst, src in zip(pin, (h, hu, hv, B)):
        np.copyto(dst, src)
    with sw.Solver(Nx, Ny) as s:
        got = s.step_host(pin[0], pin[1], pin[2], pin[3], out=tuple(pin[:3]), n_steps=2)
        assert got[0] is pin[0]
        assert same(pin[:3], want)
        assert s.time == t


@pytest.mark.parametrize("kw,dt", [({"precision": "fp32_mixed"}, None),
                                   ({"scheme": "modular"}, 1e-4)])
def test_other_forms_run_the_three_calls(gpu_lib, sw, problems, kw, dt):
    Nx, Ny = 70, 50
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=8, q_scale=0.1, b_scale=0.05)
    want, t, _ = sequence(sw, Nx, Ny, h, hu, hv, B, 2, dt, **kw)
    with sw.Solver(Nx, Ny, **kw) as s:
        got = s.step_host(h, hu, hv, B, n_steps=2, dt=dt)
        assert same(got, want)
        assert s.time == t


def test_errors(gpu_lib, sw, problems):
    L = sw._lib
    Nx, Ny = 40, 30
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=3)
    with sw.Solver(Nx, Ny) as s:
        with pytest.raises(sw.SweError) as e:
            s.step_host(h, hu, hv, None)  # the first upload needs B
        assert e.value.status == L.SWE_ERR_BAD_ARG
        bad = np.array(h)
        bad[10, 10] = np.nan
        with pytest.raises(sw.SweError) as e:
            s.step_host(bad, hu, hv, B)
        assert e.value.status == L.SWE_ERR_NONFINITE
        # the context stays usable; zero steps = upload + download with ghosts refreshed
        out = s.step_host(h, hu, hv, B, n_steps=0)
        s.upload(h, hu, hv, B)
        assert same(out, s.download())


def test_device_steps_continue_after_it(gpu_lib, sw, problems):
    """After swe_step_host the device holds the new state and its wave speed: further
    swe_step calls continue the run as if it had been one swe_step."""
    Nx, Ny = 1040, 48
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=12, q_scale=0.1, b_scale=0.05)
    want, t, dts = sequence(sw, Nx, Ny, h, hu, hv, B, 5, None)
    with sw.Solver(Nx, Ny) as s:
        s.step_host(h, hu, hv, B, n_steps=2)
        s.step(3)
        assert same(s.download(), want)
        assert s.time == t
        assert bitwise_equal(s.dt_log(3), dts[2:])


def test_slab_context_runs_the_three_calls(gpu_lib, sw, problems):
    """A slab context (ghost rows supplied by a neighbour) takes the sequential path."""
    Nx, Ny = 64, 40
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=13, q_scale=0.1, b_scale=0.05)
    want, t, _ = sequence(sw, Nx, Ny, h, hu, hv, B, 2, 1e-4, x_halo=(True, False))
    with sw.Solver(Nx, Ny, x_halo=(True, False)) as s:
        got = s.step_host(h, hu, hv, B, n_steps=2, dt=1e-4)
        assert same(got, want)
        assert s.time == t
