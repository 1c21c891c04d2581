"""On-device sanity reductions (swe_sanity) against the reference's own definitions
evaluated on the downloaded state: mass = sum h dx dy (MassConservation), h_min (Debug),
the first row-major interior cell with h < 0 (Positivity), and the energy."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_checks(h, hu, hv, B, dxdy, g):
    hi, ui, vi, bi = (a[2:-2, 2:-2] for a in (h, hu, hv, B))
    neg = np.flatnonzero(hi.ravel() < 0.0)  # row-major, i (x) outer as the reference loops
    kin = np.where(hi > 1e-8, 0.5 * (ui * ui + vi * vi) / np.where(hi > 1e-8, hi, 1.0), 0.0)
    energy = (kin + 0.5 * g * hi * hi + g * hi * bi).sum() * dxdy
    return {"mass": float(hi.sum() * dxdy), "h_min": float(hi.min()),
            "first_negative": int(neg[0]) if neg.size else -1, "energy": float(energy)}


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_sanity_matches_reference_definitions(gpu_lib, sw, problems, precision):
    Nx, Ny = 77, 53
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=4)
    h = np.array(h)
    h[2 + 30, 2 + 7] = -0.25   # two negative depths: the row-major first is (30, 7)
    h[2 + 61, 2 + 2] = -0.5
    with sw.Solver(Nx, Ny, Lx=2.0, Ly=1.5, precision=precision) as s:
        s.upload(h, hu, hv, B)
        got = s.sanity()
        dh, dhu, dhv = s.download()
        mass_totals = s.totals()[0]
    # the FP32 form holds B in FP32
    Bd = B if precision == "fp64" else np.asarray(B, dtype=np.float32).astype(np.float64)
    want = reference_checks(dh, dhu, dhv, Bd, (2.0 / Nx) * (1.5 / Ny), 9.80665)
    assert got["first_negative"] == want["first_negative"] == 30 * Ny + 7
    assert got["h_min"] == want["h_min"]
    assert abs(got["mass"] - want["mass"]) <= 1e-13 * abs(want["mass"])
    assert got["mass"] == mass_totals
    assert abs(got["energy"] - want["energy"]) <= 1e-12 * abs(want["energy"])


def test_sanity_after_steps_sees_the_positivity_floor(gpu_lib, sw, problems):
    B, _ = problems.gaussian_sum_bathymetry(96, 64, n=6, seed=3, bc="transmissive")
    h, hu, hv = problems.dam_break(B)
    with sw.Solver(96, 64, bc="transmissive") as s:
        s.upload(h, hu, hv, B)
        m0 = s.sanity()["mass"]
        s.step(20)
        r = s.sanity()
        dh, dhu, dhv = s.download()
    assert r["first_negative"] == -1 and r["h_min"] >= 0.0
    assert r["h_min"] == float(dh[2:-2, 2:-2].min())
    assert abs(r["mass"] - m0) <= 1e-2 * m0  # transmissive walls: mass leaves slowly
