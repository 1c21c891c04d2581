"""The C restatement of the modular SerialSolver (oracle/swe_modular.c) against the
reference itself: against the committed fixtures in tests/golden/modular_20x14.npz
(generated by tests/golden/make_golden.py from the reference's own SerialSolver), and,
where the reference is compiled here (oracle/_ref), live on further inputs."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden", "modular_20x14.npz")
COMBOS = [(r, s, b) for r in (0, 1) for s in (0, 1, 2) for b in (0, 1)]


def same(a, b):
    """Bitwise, except that NaNs match any NaN (their payload and sign are the CPU's)."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    na, nb = np.isnan(a), np.isnan(b)
    return a.shape == b.shape and np.array_equal(na, nb) and np.array_equal(
        a[~na].view(np.uint64), b[~nb].view(np.uint64))


@pytest.mark.parametrize("tag", ["wet", "dry"])
@pytest.mark.parametrize("recon,riemann,bathy", COMBOS)
def test_port_matches_modular_golden(port, tag, recon, riemann, bathy):
    d = np.load(GOLDEN)
    m = json.loads(str(d["meta"]))
    p = port.grid(m["Nx"], m["Ny"], m["Lx"], m["Ly"], cfl=m["cfl"])
    dt, dt_guard = d[f"{tag}_dt"]
    got_guard, st = port.modular_stable_dt(p, d[f"{tag}_h"], d[f"{tag}_hu"], d[f"{tag}_hv"])
    assert st == 0 and got_guard == dt_guard
    h, hu, hv, t, st = port.modular_run(p, recon, riemann, bathy, d[f"{tag}_h"], d[f"{tag}_hu"],
                                        d[f"{tag}_hv"], d[f"{tag}_B"], m["steps"], dt)
    key = f"{tag}_r{recon}_s{riemann}_b{bathy}"
    assert st == int(d[key + "_status"][0])
    for a, b in zip((h, hu, hv), d[key]):
        assert same(a, b)


ref = pytest.importorskip("oracle.ref")
needs_ref = pytest.mark.skipif(not ref.available(), reason="oracle/_ref not built")


@needs_ref
@pytest.mark.parametrize("seed,Nx,Ny,dry", [(1, 16, 27, 0.0), (2, 31, 12, 0.15), (4, 9, 9, 0.3)])
@pytest.mark.parametrize("recon,riemann,bathy", COMBOS)
def test_port_matches_reference_modular(port, problems, seed, Nx, Ny, dry, recon, riemann,
                                        bathy):
    Lx, Ly = 0.7 + 0.1 * seed, 1.0
    h, hu, hv, B = (np.array(a) for a in problems.random_state(Nx, Ny, seed=seed, dry_frac=dry))
    p = port.grid(Nx, Ny, Lx, Ly)
    port.fill_ghosts(p, h, hu, hv)
    port.fill_scalar_ghosts(p, B)
    m = h < 1e-7
    hu[m] = 0.0
    hv[m] = 0.0
    dt_ref, st_ref = ref.modular_stable_dt(Nx, Ny, h, hu, hv, Lx, Ly)
    dt_port, st_port = port.modular_stable_dt(p, h, hu, hv)
    assert (st_port, dt_port) == (st_ref, dt_ref)
    a = port.modular_run(p, recon, riemann, bathy, h, hu, hv, B, 10, 0.6 * dt_ref)
    b = ref.modular_run(Nx, Ny, recon, riemann, bathy, h, hu, hv, B, 10, 0.6 * dt_ref, Lx, Ly)
    assert a[4] == b[3]
    for x, y in zip(a[:3], b[:3]):
        assert same(x, y)


@needs_ref
@pytest.mark.parametrize("recon", [0, 1])
def test_hll_failure_and_cfl_guard_statuses(port, problems, recon):
    """A NaN depth makes HLL's speeds NaN: the reference throws "HLL could not provide
    dissipation speed." (status 2 in both); h < 0 makes the CFL guard throw (status 1)."""
    Nx, Ny = 12, 10
    h, hu, hv, B = (np.array(a) for a in problems.random_state(Nx, Ny, seed=9))
    p = port.grid(Nx, Ny)
    port.fill_ghosts(p, h, hu, hv)
    h[6, 5] = np.nan
    a = port.modular_run(p, recon, 0, 0, h, hu, hv, B, 2, 1e-4)
    b = ref.modular_run(Nx, Ny, recon, 0, 0, h, hu, hv, B, 2, 1e-4)
    assert a[4] == b[3] == 2
    h[6, 5] = -0.5
    assert port.modular_stable_dt(p, h, hu, hv)[1] == ref.modular_stable_dt(Nx, Ny, h, hu, hv)[1] == 1
