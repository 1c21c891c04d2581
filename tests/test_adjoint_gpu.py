"""GPU discrete adjoint (swe_adjoint_gauge) against (a) the CPU reference adjoint of
tests/cpp/adjoint_ref.cpp, (b) central finite differences of the CPU oracle (the
reference's algorithm) along random smooth directions, relative agreement 1e-6,
(c) itself under every checkpoint budget (bitwise), and (d) through the
torch.autograd.Function.

The scheme is only piecewise smooth: minmod switches between its slopes wherever they
are equal in magnitude (inflection lines), and max(b-, b+) and the HLL wave-speed min/max
switch too, so J has kinks at every scale.  A central difference straddles some of them
with a probability proportional to eps: at eps = 1e-6 the agreement is about 1e-6 in the
median and 3e-5 at worst on these cases, at eps = 1e-7 about 1e-7.  The checks use
eps = 1e-7 against the 1e-6 bar; rounding noise in J stays near 1e-10 relative there.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_adjoint_cpu import smooth_case, smooth_direction

pytestmark = pytest.mark.gpu

FD_REL = 1e-6
FD_EPS = 1e-7


def setup(problems, Nx, Ny, bc, steps, seed):
    h, hu, hv, B, rng = smooth_case(problems, Nx, Ny, bc, seed)
    ng = 7
    gauges = np.stack([rng.integers(0, Nx, ng), rng.integers(0, Ny, ng)], axis=1)
    obs = 1.0 + 0.01 * rng.standard_normal((steps, ng))
    return h, hu, hv, B, gauges, obs, rng


def oracle_J(port, p, h, hu, hv, B, steps, dt, gauges, obs):
    """J from the CPU oracle, one step at a time."""
    a = [np.array(x, copy=True) for x in (h, hu, hv)]
    ws = port.Workspace(p)
    J = 0.0
    for n in range(steps):
        _, _, st = ws.run_inplace(a[0], a[1], a[2], B, 1, dt)
        assert st == 0
        r = a[0][gauges[:, 0] + 2, gauges[:, 1] + 2] - obs[n]
        J += float((r * r).sum())
    ws.close()
    return J


def gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, bc, snapshots=None,
                precision="fp64"):
    with sw.Solver(Nx, Ny, bc=bc, precision=precision) as s:
        s.upload(h, hu, hv, B)
        r = sw.adjoint.gauge_misfit_gradient(s, steps, dt, gauges, obs, snapshots)
        out = s.download()
    r["state_after"] = out
    return r


@pytest.mark.parametrize("bc", [0, 1], ids=["reflecting", "transmissive"])
def test_gpu_adjoint_matches_cpu_reference_adjoint(gpu_lib, sw, problems, bc):
    import adjref
    Nx, Ny, steps, dt = 24, 20, 10, 1e-3
    h, hu, hv, B, gauges, obs, _ = setup(problems, Nx, Ny, bc, steps, seed=3 + bc)
    r = gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, bc)
    J, gh, ghu, ghv, gB = adjref.run(Nx, Ny, h, hu, hv, B, steps, dt, gauges[:, 0],
                                     gauges[:, 1], obs, bc=bc)
    assert abs(r["J"] - J) <= 1e-12 * abs(J)
    for got, want in zip((r["grad_h"], r["grad_hu"], r["grad_hv"], r["grad_B"]),
                         (gh, ghu, ghv, gB)):
        scale = np.abs(want[2:-2, 2:-2]).max()
        assert np.abs(got[2:-2, 2:-2] - want[2:-2, 2:-2]).max() <= 1e-11 * scale
    # the context's state is left as uploaded
    assert np.array_equal(r["state_after"][0][2:-2, 2:-2], h[2:-2, 2:-2])


@pytest.mark.parametrize("bc", [0, 1], ids=["reflecting", "transmissive"])
def test_gpu_adjoint_matches_oracle_finite_differences(gpu_lib, sw, port, problems, bc):
    Nx, Ny, steps, dt = 32, 28, 16, 1e-3
    h, hu, hv, B, gauges, obs, rng = setup(problems, Nx, Ny, bc, steps, seed=11 + bc)
    r = gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, bc)
    p = port.grid(Nx, Ny, bc=bc)
    J0 = oracle_J(port, p, h, hu, hv, B, steps, dt, gauges, obs)
    assert abs(r["J"] - J0) <= 1e-12 * abs(J0)
    bcs = "reflecting" if bc == 0 else "transmissive"
    eps = FD_EPS
    for trial in range(4):
        d = [smooth_direction(problems, Nx, Ny, rng) for _ in range(4)]
        dB = d[3].copy()
        problems.fill_scalar_ghosts(dB, bcs)

        def J_at(s):
            return oracle_J(port, p, h + s * d[0], hu + s * d[1], hv + s * d[2], B + s * dB,
                            steps, dt, gauges, obs)

        fd = (J_at(eps) - J_at(-eps)) / (2 * eps)
        ad = sum(float((g[2:-2, 2:-2] * x[2:-2, 2:-2]).sum()) for g, x in
                 zip((r["grad_h"], r["grad_hu"], r["grad_hv"], r["grad_B"]), d))
        assert abs(fd - ad) <= FD_REL * abs(fd), (trial, fd, ad)


def test_checkpoint_budget_does_not_change_the_gradient(gpu_lib, sw, problems):
    Nx, Ny, steps, dt = 20, 16, 13, 1e-3
    h, hu, hv, B, gauges, obs, _ = setup(problems, Nx, Ny, 0, steps, seed=23)
    base = gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, 0, snapshots=steps)
    for snaps in (0, 1, 2, 4, "tape", "segments"):
        r = gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, 0, snapshots=snaps)
        assert r["J"] == base["J"]
        for k in ("grad_h", "grad_hu", "grad_hv", "grad_B"):
            assert np.array_equal(r[k], base[k]), (snaps, k)


@pytest.mark.parametrize("steps", [1, 2, 3, 4, 9])
def test_segmented_schedule_edge_lengths(gpu_lib, sw, problems, steps):
    # one segment, segments of one step, a last segment of one step, whole segments only:
    # the first sweep stops at the last segment's start, which is taped straight away
    Nx, Ny, dt = 18, 14, 1e-3
    h, hu, hv, B, gauges, obs, _ = setup(problems, Nx, Ny, 0, steps, seed=31 + steps)
    base = gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, 0, snapshots=steps)
    for snaps in ("tape", "segments"):
        r = gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, 0, snapshots=snaps)
        assert r["J"] == base["J"]
        for k in ("grad_h", "grad_hu", "grad_hv", "grad_B"):
            assert np.array_equal(r[k], base[k]), (snaps, k)


def test_autograd_function_gradients(gpu_lib, sw, port, problems):
    import torch
    Nx, Ny, steps, dt = 24, 24, 12, 1e-3
    rng = np.random.default_rng(5)
    Bg, _ = problems.gaussian_sum_bathymetry(Nx, Ny, n=4, rng=rng, width=(0.15, 0.3),
                                             amp=(-0.1, 0.1))
    B = Bg[2:-2, 2:-2] + 1e-3 * rng.standard_normal((Nx, Ny))
    x = problems.centres(Nx)[2:-2, None]
    y = problems.centres(Ny)[None, 2:-2]
    eta0 = 1.0 + 0.03 * np.exp(-((x - 0.5) ** 2 + (y - 0.45) ** 2) / 0.03)
    eta0 = eta0 + 1e-3 * rng.standard_normal((Nx, Ny))
    gauges = np.stack([rng.integers(0, Nx, 6), rng.integers(0, Ny, 6)], axis=1)
    obs = 1.0 + 0.01 * rng.standard_normal((steps, 6))
    te = torch.tensor(eta0, requires_grad=True)
    tb = torch.tensor(B, requires_grad=True)
    J = sw.adjoint.GaugeMisfit.apply(te, tb, steps, dt, gauges, obs)
    J.backward()
    p = port.grid(Nx, Ny)

    def J_np(e, b):
        h, hu, hv, Bg2 = sw.adjoint.ghosted_state(e, b)
        return oracle_J(port, p, h, hu, hv, Bg2, steps, dt, gauges, obs)

    assert abs(J.item() - J_np(eta0, B)) <= 1e-12 * J.item()
    eps = FD_EPS
    for trial in range(3):
        de = smooth_direction(problems, Nx, Ny, rng)[2:-2, 2:-2]
        db = smooth_direction(problems, Nx, Ny, rng)[2:-2, 2:-2]
        fd = (J_np(eta0 + eps * de, B + eps * db) - J_np(eta0 - eps * de, B - eps * db)) / (2 * eps)
        ad = float((te.grad.numpy() * de).sum() + (tb.grad.numpy() * db).sum())
        assert abs(fd - ad) <= FD_REL * abs(fd), (trial, fd, ad)


# FP32-mixed adjoint: the FP32 forward trajectory and the interface derivative evaluated
# in FP32, against the FP64 adjoint of the same problem.  Measured on these cases: J
# within about 1e-6, directional derivatives along smooth directions within about 1e-5
# (the bar below is 10x that); the gradient fields differ more where a minmod or
# wave-speed branch flips between the two trajectories.  The FP32 interface VJP recomputes
# its branch decisions in its own formulation (IEEE reciprocals, the classic HLL form),
# not the FP32 forward's (approximate reciprocals, the flux-difference form), so a near-tie
# can be decided differently by the two.  When the forward's roundings were pinned to an
# explicit order, one direction of the transmissive case moved from 4e-7 to 8e-4 while the
# FP64 adjoint of the same inputs rounded to FP32 moved by 6e-7: a single decision of that
# kind, not rounding of the state.  The bar is therefore on the median over eight
# directions, with the largest held to 2e-3.
FP32_J_REL = 1e-5
FP32_DIR_REL = 1e-4
FP32_DIR_MAX = 2e-3


@pytest.mark.parametrize("bc", [0, 1], ids=["reflecting", "transmissive"])
def test_fp32_adjoint_agrees_with_fp64_adjoint(gpu_lib, sw, problems, bc):
    Nx, Ny, steps, dt = 32, 28, 16, 1e-3
    h, hu, hv, B, gauges, obs, rng = setup(problems, Nx, Ny, bc, steps, seed=31 + bc)
    r64 = gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, bc)
    r32 = gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, bc,
                      precision="fp32_mixed")
    assert abs(r32["J"] - r64["J"]) <= FP32_J_REL * abs(r64["J"])
    f32 = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    Br = f32(B)
    r64r = gpu_adjoint(sw, f32(h + Br) - Br, f32(hu), f32(hv), Br, Nx, Ny, steps, dt, gauges,
                       obs, bc)
    rel, rel_rounded = [], []
    for trial in range(8):
        d = [smooth_direction(problems, Nx, Ny, rng) for _ in range(4)]
        a64, a32, a64r = (sum(float((g[2:-2, 2:-2] * x[2:-2, 2:-2]).sum()) for g, x in
                              zip((r["grad_h"], r["grad_hu"], r["grad_hv"], r["grad_B"]), d))
                          for r in (r64, r32, r64r))
        rel.append(abs(a32 - a64) / abs(a64))
        rel_rounded.append(abs(a64r - a64) / abs(a64))
    print("fp32 adjoint vs fp64:", " ".join(f"{x:.1e}" for x in rel),
          "| fp64 of fp32-rounded inputs:", " ".join(f"{x:.1e}" for x in rel_rounded))
    assert np.median(rel) <= FP32_DIR_REL, rel
    assert max(rel) <= FP32_DIR_MAX, rel


def test_fp32_checkpoint_budget_does_not_change_the_gradient(gpu_lib, sw, problems):
    Nx, Ny, steps, dt = 20, 16, 13, 1e-3
    h, hu, hv, B, gauges, obs, _ = setup(problems, Nx, Ny, 0, steps, seed=29)
    base = gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, 0, snapshots=steps,
                       precision="fp32_mixed")
    for snaps in (0, 3, "tape", "segments"):
        r = gpu_adjoint(sw, h, hu, hv, B, Nx, Ny, steps, dt, gauges, obs, 0, snapshots=snaps,
                        precision="fp32_mixed")
        assert r["J"] == base["J"]
        for k in ("grad_h", "grad_hu", "grad_hv", "grad_B"):
            assert np.array_equal(r[k], base[k]), (snaps, k)


# ---- The finite-difference check at the adjoint workload's grid ---------------------------
# 1024^2, 16 seeded Gaussians of bed, eta0 = 1 + 8 seeded bumps, 64 gauges, observations
# from a forward run with a perturbed surface and bed; 20 steps of the CPU oracle (the
# reference's algorithm) per evaluation, central differences with eps = 1e-6 along 16
# random smooth directions in the initial depth and the bed.
#
# Far from the bumps the surface and the bed are flat to rounding: minmod there compares
# slopes of ~1e-16 and max(b-, b+) beds of ~1e-30, so the evaluation point itself sits on
# kinks that any perturbation above rounding crosses; a central difference then averages
# the one-sided derivatives, while the adjoint takes the branch the forward took.  On this
# problem the agreement is ~1e-5 (median) relative to |FD| and ~1e-5 relative to the
# projection's absolute terms.  With 1e-3 noise in the surface and the bed, which moves
# those ties away from rounding level, the same check agrees within 1e-6: in the median
# relative to |FD|, and for every direction relative to the projection's absolute terms
# (a direction whose projection nearly cancels has |FD| far below its terms; one of the
# 16 here is 3e-5 relative to |FD| and 3e-8 relative to its terms).
def adjoint_workload(problems, n, steps, noise, seed=2033):
    rng = np.random.default_rng(seed)
    B, _ = problems.gaussian_sum_bathymetry(n, n, n=16, rng=rng, bc="reflecting")
    bumps, _ = problems.gaussian_sum_bathymetry(n, n, n=8, rng=rng, width=(0.02, 0.1),
                                                amp=(-0.05, 0.05), bc="reflecting")
    if noise:
        B = B + noise * rng.standard_normal(B.shape)
        problems.fill_scalar_ghosts(B, "reflecting")
        bumps = bumps + noise * rng.standard_normal(B.shape)
    h = np.maximum(0.0, 1.0 + bumps - B)
    gauges = np.stack([rng.integers(0, n, 64), rng.integers(0, n, 64)], axis=1)
    return h, B, bumps, gauges, rng


@pytest.mark.parametrize("noise", [0.0, 1e-3], ids=["stated", "noise-1e-3"])
def test_adjoint_against_oracle_fd_at_1024(gpu_lib, sw, port, problems, noise):
    n, steps, eps = 1024, 20, 1e-6
    h, B, bumps, gauges, rng = adjoint_workload(problems, n, steps, noise)
    z = np.zeros_like(h)
    with sw.Solver(n, n) as s:
        s.upload(h, z, z, B)
        dt = 0.5 * s.stable_dt()
        s.upload(np.maximum(0.0, 1.0 + 1.05 * bumps - 1.02 * B), z, z, 1.02 * B)
        obs = sw.adjoint.gauge_series(s, steps, dt, gauges)
        s.upload(h, z, z, B)
        r = sw.adjoint.gauge_misfit_gradient(s, steps, dt, gauges, obs, "tape")
        J_gpu, _ = sw.adjoint.gauge_misfit(s, steps, dt, gauges, obs)
    p = port.grid(n, n)
    J0 = oracle_J(port, p, h, z, z, B, steps, dt, gauges, obs)
    assert abs(J0 - r["J"]) <= 1e-12 * J0
    assert J_gpu == r["J"]  # the objective-only call: bitwise the gradient call's J
    rel, rel_abs = [], []
    for _ in range(16):
        dh = problems.gaussian_sum_bathymetry(n, n, n=4, rng=rng, width=(0.1, 0.3),
                                              amp=(-1.0, 1.0))[0]
        dB = problems.gaussian_sum_bathymetry(n, n, n=4, rng=rng, width=(0.1, 0.3),
                                              amp=(-1.0, 1.0), bc="reflecting")[0]
        dh = np.where(h > 0, dh, 0.0)
        fd = (oracle_J(port, p, h + eps * dh, z, z, B + eps * dB, steps, dt, gauges, obs) -
              oracle_J(port, p, h - eps * dh, z, z, B - eps * dB, steps, dt, gauges, obs)) / (2 * eps)
        terms = (r["grad_h"] * dh, r["grad_B"] * dB)
        ad = float(sum(t.sum() for t in terms))
        rel.append(abs(fd - ad) / abs(fd))
        rel_abs.append(abs(fd - ad) / float(sum(np.abs(t).sum() for t in terms)))
    print(f"noise {noise}: |FD - adjoint| / |FD| median {np.median(rel):.3g} max {max(rel):.3g}; "
          f"/ abs terms max {max(rel_abs):.3g}")
    if noise:
        assert np.median(rel) <= FD_REL, rel
        assert max(rel_abs) <= FD_REL, rel_abs
    else:
        assert np.median(rel) <= 1e-4 and max(rel) <= 1e-3, rel
        assert max(rel_abs) <= 5e-5, rel_abs
