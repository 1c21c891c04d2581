"""The modular scheme (SerialSolver's arithmetic) on the GPU, bitwise against the
reference's own outputs (tests/golden/modular_20x14.npz, generated from SerialSolver
itself) and against the oracle on larger, ragged grids, for every reconstruction x
Riemann solver, with and without bathymetry."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden", "modular_20x14.npz")
COMBOS = [(r, s, b) for r in (0, 1) for s in (0, 1, 2) for b in (0, 1)]
RECON = ("PiecewiseConst", "MUSCL")
RIEMANN = ("HLL", "Rusanov", "ROE")


def same(a, b):
    """Bitwise, except that NaNs match any NaN (their payload and sign are the CPU's)."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    na, nb = np.isnan(a), np.isnan(b)
    return a.shape == b.shape and np.array_equal(na, nb) and np.array_equal(
        a[~na].view(np.uint64), b[~nb].view(np.uint64))


def modular(sw, Nx, Ny, Lx, Ly, recon, riemann, bathy):
    return sw.Solver(Nx, Ny, Lx=Lx, Ly=Ly, scheme="modular", reconstruction=RECON[recon],
                     riemann=RIEMANN[riemann], bathymetry=bool(bathy))


@pytest.mark.parametrize("tag", ["wet", "dry"])
@pytest.mark.parametrize("recon,riemann,bathy", COMBOS)
def test_modular_matches_reference_golden(gpu_lib, sw, tag, recon, riemann, bathy):
    d = np.load(GOLDEN)
    m = json.loads(str(d["meta"]))
    dt, dt_guard = d[f"{tag}_dt"]
    key = f"{tag}_r{recon}_s{riemann}_b{bathy}"
    want_status = int(d[key + "_status"][0])
    with modular(sw, m["Nx"], m["Ny"], m["Lx"], m["Ly"], recon, riemann, bathy) as s:
        s.upload(d[f"{tag}_h"], d[f"{tag}_hu"], d[f"{tag}_hv"], d[f"{tag}_B"])
        assert s.stable_dt() == dt_guard  # time_utils.hpp's guard, bitwise
        if want_status:
            with pytest.raises(sw.SweError) as e:
                s.step(m["steps"], dt)
            assert e.value.status == sw._lib.SWE_ERR_NONFINITE
            assert ("HLL could not" if want_status == 2 else "non-finite") in str(e.value)
            return
        s.step(m["steps"], dt)
        got = s.download()
    for a, b in zip(got, d[key]):
        assert same(a, b)


@pytest.mark.parametrize("recon,riemann,bathy", COMBOS)
def test_modular_matches_oracle_ragged(gpu_lib, sw, port, problems, recon, riemann, bathy):
    """101 x 77: ragged last tiles in x (8-row tiles) and y (32-column tiles)."""
    Nx, Ny, Lx, Ly, steps = 101, 77, 1.0, 0.8, 12
    h, hu, hv, B = (np.array(a) for a in problems.random_state(Nx, Ny, seed=31, dry_frac=0.02))
    p = port.grid(Nx, Ny, Lx, Ly)
    port.fill_ghosts(p, h, hu, hv)
    port.fill_scalar_ghosts(p, B)
    dry = h < 1e-7
    hu[dry] = 0.0
    hv[dry] = 0.0
    dt_guard, st = port.modular_stable_dt(p, h, hu, hv)
    assert st == 0
    dt = 0.5 * dt_guard
    oh, ohu, ohv, ot, ost = port.modular_run(p, recon, riemann, bathy, h, hu, hv, B, steps, dt)
    with modular(sw, Nx, Ny, Lx, Ly, recon, riemann, bathy) as s:
        s.upload(h, hu, hv, B)
        if ost:
            with pytest.raises(sw.SweError):
                s.step(steps, dt)
            return
        t = s.step(steps, dt)
        got = s.download()
    assert t == ot
    for a, b in zip(got, (oh, ohu, ohv)):
        assert same(a, b)


@pytest.mark.parametrize("recon,riemann", [(r, s) for r in (0, 1) for s in (0, 1, 2)])
def test_modular_lake_at_rest(gpu_lib, sw, port, problems, recon, riemann):
    """A wet lake at rest over bumps stays at rest to rounding (about 1e-15: the
    reference's SerialSolver is balanced only to rounding, unlike the fused scheme's
    exact zero), bitwise as the oracle."""
    Nx = Ny = 64
    B, _ = problems.gaussian_sum_bathymetry(Nx, Ny, n=5, seed=2, amp=(-0.3, 0.4))
    h, hu, hv = problems.lake_at_rest(B, 1.0)
    p = port.grid(Nx, Ny)
    dt = 0.5 * port.modular_stable_dt(p, h, hu, hv)[0]
    oh, ohu, ohv, _, st = port.modular_run(p, recon, riemann, 1, h, hu, hv, B, 50, dt)
    assert st == 0
    with modular(sw, Nx, Ny, 1.0, 1.0, recon, riemann, 1) as s:
        s.upload(h, hu, hv, B)
        s.step(50, dt)
        got = s.download()
    for a, b in zip(got, (oh, ohu, ohv)):
        assert same(a, b)
    assert max(np.abs(got[1][2:-2, 2:-2]).max(), np.abs(got[2][2:-2, 2:-2]).max()) < 1e-13


def test_modular_options_and_errors(gpu_lib, sw, problems):
    L = sw._lib
    with pytest.raises(sw.SweError) as e:
        sw.Solver(16, 16, scheme="modular", precision="fp32_mixed")
    assert e.value.status == L.SWE_ERR_UNSUPPORTED
    with pytest.raises(sw.SweError) as e:
        sw.Solver(16, 16, scheme="modular", bc="transmissive")
    assert e.value.status == L.SWE_ERR_UNSUPPORTED
    h, hu, hv, B = problems.random_state(16, 16, seed=1)
    with modular(sw, 16, 16, 1.0, 1.0, 1, 1, 0) as s:
        s.upload(h, hu, hv, B)
        with pytest.raises(sw.SweError) as e:
            s.step(1)  # adaptive dt: the Serial backend has none
        assert e.value.status == L.SWE_ERR_UNSUPPORTED
        h2 = np.array(h)
        h2[5, 5] = -1.0
        s.upload(h2, hu, hv, B)
        with pytest.raises(sw.SweError) as e:
            s.stable_dt()
        assert "h <= 0" in str(e.value)
