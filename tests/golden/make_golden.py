"""Generates the golden fixtures in this directory by running the reference itself.

Requires oracle/_ref (``make -C oracle ref``, which compiles the reference's own
HPC_solver / omp_solver from its sources).  Inputs come from
shallow-water_gb300/problems.py; they are stored in the fixtures (small cases) or
pinned by their SHA-256 (the full 256^2 parity case), so the fixtures do not depend
on the platform's exp().

    python tests/golden/make_golden.py [--modular-only]
"""
from __future__ import annotations

import hashlib
import importlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
P = importlib.import_module("shallow-water_gb300.problems")
from oracle import ref  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def case_config0(variant):
    """256^2 Gaussian hump over flat B = 0, reflecting walls, CFL 0.45 fixed dt, 1000 steps."""
    N = 256
    h, hu, hv, B = P.gauss_hump(N, N)
    dt = ref.stable_dt(N, N, h, hu, hv, cfl=0.45, variant=variant)
    o = ref.run(N, N, h, hu, hv, B, 1000, dt_fixed=dt, cfl=0.45, bc=0, variant=variant)
    assert o[5] == 0
    return {
        "N": N, "steps": 1000, "dt": dt, "g": ref.gravity(variant), "bc": 0, "cfl": 0.45,
        "input_sha256": {"h": sha(h), "hu": sha(hu), "hv": sha(hv), "B": sha(B)},
        "output_sha256": {"h": sha(o[0]), "hu": sha(o[1]), "hv": sha(o[2])},
        "output_stats": {k: [float(a.sum()), float(np.abs(a).max())]
                         for k, a in zip(("h", "hu", "hv"), o[:3])},
        "t_end": o[4],
    }


def small_cases():
    cases = {}
    # rough random state with dry / sub-floor cells, reflecting walls, adaptive dt
    h, hu, hv, B = P.random_state(40, 24, seed=7, dry_frac=0.08)
    cases["random_dry_40x24"] = dict(Nx=40, Ny=24, Lx=1.0, Ly=0.75, cfl=0.3, bc=0, steps=30,
                                     dt_fixed=0.0, h=h, hu=hu, hv=hv, B=B)
    # dam break over seeded Gaussian bathymetry, transmissive walls, adaptive dt
    B, _ = P.gaussian_sum_bathymetry(48, 40, n=16, seed=3, bc="transmissive")
    h, hu, hv = P.dam_break(B)
    cases["dambreak_trans_48x40"] = dict(Nx=48, Ny=40, Lx=1.0, Ly=1.0, cfl=0.45, bc=1, steps=40,
                                         dt_fixed=0.0, h=h, hu=hu, hv=hv, B=B)
    # lake at rest over emerged + submerged bumps, reflecting walls, fixed dt
    B, _ = P.gaussian_sum_bathymetry(32, 32, n=6, seed=11, amp=(-0.4, 1.3))
    h, hu, hv = P.lake_at_rest(B, 1.0)
    cases["lake_island_32"] = dict(Nx=32, Ny=32, Lx=1.0, Ly=1.0, cfl=0.45, bc=0, steps=60,
                                   dt_fixed=2.0e-3, h=h, hu=hu, hv=hv, B=B)
    # odd sizes, fixed dt
    h, hu, hv, B = P.random_state(17, 33, seed=5, q_scale=0.1, b_scale=0.05)
    cases["odd_17x33"] = dict(Nx=17, Ny=33, Lx=0.5, Ly=1.0, cfl=0.45, bc=0, steps=25,
                              dt_fixed=5.0e-4, h=h, hu=hu, hv=hv, B=B)
    out = {}
    for name, c in cases.items():
        o = ref.run(c["Nx"], c["Ny"], c["h"], c["hu"], c["hv"], c["B"], c["steps"],
                    dt_fixed=c["dt_fixed"], Lx=c["Lx"], Ly=c["Ly"], cfl=c["cfl"], bc=c["bc"])
        assert o[5] == 0, name
        out[name] = dict(c, h_out=o[0], hu_out=o[1], hv_out=o[2], dts=o[3], t_end=o[4])
    return out


def modular_cases():
    """The modular SerialSolver (every reconstruction x Riemann solver, with and without
    bathymetry) on a wet and a partly dry random state, 8 fixed-dt steps at half the
    modular CFL limit; reflecting walls (the only ones it has)."""
    from oracle import port
    Nx, Ny, Lx, Ly = 20, 14, 1.1, 0.8
    out = {}
    for tag, dry in (("wet", 0.0), ("dry", 0.1)):
        h, hu, hv, B = (np.array(a) for a in P.random_state(Nx, Ny, seed=17, dry_frac=dry))
        p = port.grid(Nx, Ny, Lx, Ly)
        port.fill_ghosts(p, h, hu, hv)
        port.fill_scalar_ghosts(p, B)
        m = h < 1e-7
        hu[m] = 0.0
        hv[m] = 0.0
        dt_guard, st = ref.modular_stable_dt(Nx, Ny, h, hu, hv, Lx, Ly)
        assert st == 0
        dt = 0.5 * dt_guard
        out[f"{tag}_h"], out[f"{tag}_hu"], out[f"{tag}_hv"], out[f"{tag}_B"] = h, hu, hv, B
        out[f"{tag}_dt"] = np.array([dt, dt_guard])
        for recon in (0, 1):
            for riemann in (0, 1, 2):
                for bathy in (0, 1):
                    o = ref.modular_run(Nx, Ny, recon, riemann, bathy, h, hu, hv, B, 8, dt,
                                        Lx, Ly)
                    key = f"{tag}_r{recon}_s{riemann}_b{bathy}"
                    out[key] = np.stack(o[:3])
                    out[key + "_status"] = np.array([o[3]])
    meta = dict(Nx=Nx, Ny=Ny, Lx=Lx, Ly=Ly, steps=8, cfl=0.45)
    np.savez_compressed(os.path.join(HERE, "modular_20x14.npz"), meta=json.dumps(meta), **out)


def main():
    assert ref.available() and ref.available("g981"), "build oracle/_ref first: make -C oracle ref"
    if "--modular-only" in sys.argv:
        modular_cases()
        return
    meta = {"config0_g980665": case_config0("g980665"), "config0_g981": case_config0("g981")}
    with open(os.path.join(HERE, "config0_256.json"), "w") as f:
        json.dump(meta, f, indent=1)
    for name, c in small_cases().items():
        arrays = {k: v for k, v in c.items() if isinstance(v, np.ndarray)}
        scalars = {k: v for k, v in c.items() if not isinstance(v, np.ndarray)}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(scalars), **arrays)
    modular_cases()
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
