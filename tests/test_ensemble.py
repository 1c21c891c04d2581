"""Batched ensembles on the GPU: every instance, advanced in one launch per stage with
its own CFL dt, equals the CPU oracle run on that instance alone (FP64: bitwise; FP32:
bitwise equal to the single-grid FP32 path), for every schedule the autotuner can pick."""
from __future__ import annotations

import pytest

from conftest import bitwise_equal

pytestmark = pytest.mark.gpu

SIZES = [(17, 33), (64, 64), (40, 96), (128, 32), (2, 2), (96, 130)]


def members(problems, sizes, seed=3):
    out = []
    for k, (nx, ny) in enumerate(sizes):
        h, hu, hv, B = problems.random_state(nx, ny, seed=seed + k, q_scale=0.1, b_scale=0.05)
        out.append((h, hu, hv, B))
    return out


def test_fp64_ensemble_matches_oracle_per_instance(gpu_lib, sw, port, problems):
    mem = members(problems, SIZES)
    with sw.Ensemble(SIZES, cfl=0.3) as ens:
        for q, m in enumerate(mem):
            ens.upload(q, *m)
        ens.step(12)
        times = ens.times()
        for q, (nx, ny) in enumerate(SIZES):
            ref = port.run(port.grid(nx, ny, cfl=0.3), *mem[q], 12, 0.0)
            out = ens.download(q)
            for k in range(3):
                assert bitwise_equal(out[k], ref[k]), (q, k)
            assert times[q] == ref[4]


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_every_schedule_gives_identical_results(gpu_lib, sw, problems, precision):
    mem = members(problems, SIZES, seed=11)
    shapes = (["8x32", "8x16", "4x64", "strip"] if precision == "fp64"
              else ["8x32", "16x32", "8x64", "cols"])
    results = []
    for shape in shapes:
        for grid in (0, 152, 608):
            with sw.Ensemble(SIZES, cfl=0.3, precision=precision) as ens:
                ens.set_schedule(shape, grid)
                for q, m in enumerate(mem):
                    ens.upload(q, *m)
                ens.step(4)
                ens.step(3)
                results.append([ens.download(q) for q in range(len(SIZES))])
    for r in results[1:]:
        for q in range(len(SIZES)):
            for k in range(3):
                assert bitwise_equal(r[q][k], results[0][q][k])


def test_fp32_ensemble_equals_single_grid(gpu_lib, sw, problems):
    mem = members(problems, SIZES, seed=5)
    with sw.Ensemble(SIZES, cfl=0.3, precision="fp32_mixed") as ens:
        for q, m in enumerate(mem):
            ens.upload(q, *m)
        ens.step(10)
        outs = [ens.download(q) for q in range(len(SIZES))]
        t = ens.times()
    for q, (nx, ny) in enumerate(SIZES):
        with sw.Solver(nx, ny, cfl=0.3, precision="fp32_mixed") as s:
            s.upload(*mem[q])
            s.step(10)
            ref = s.download()
            for k in range(3):
                assert bitwise_equal(outs[q][k], ref[k]), (q, k)
            assert t[q] == s.time


def test_tuner_restores_state_and_picks_a_schedule(gpu_lib, sw, port, problems, tmp_path):
    mem = members(problems, SIZES, seed=21)
    cache = str(tmp_path / "tune.json")
    with sw.Ensemble(SIZES, cfl=0.3) as ens:
        for q, m in enumerate(mem):
            ens.upload(q, *m)
        res = ens.tune(steps=1, cache=cache)
        assert res["shape"] in ("8x32", "8x16", "4x64", "strip") and res["ms_per_step"] > 0
        assert not res["cached"]
        ens.step(5)
        for q, (nx, ny) in enumerate(SIZES):
            ref = port.run(port.grid(nx, ny, cfl=0.3), *mem[q], 5, 0.0)
            out = ens.download(q)
            assert bitwise_equal(out[0], ref[0]) and bitwise_equal(out[2], ref[2])
    with sw.Ensemble(SIZES, cfl=0.3) as ens2:
        assert ens2.tune(steps=1, cache=cache)["cached"]


def test_config3_style_members_fixed_and_adaptive(gpu_lib, sw, port, problems):
    specs = problems.ensemble_instances(count=5, sizes=(32, 64, 128), seed=7)
    mem = [problems.ensemble_member(n, s) for n, s in specs]
    sizes = [(n, n) for n, _ in specs]
    with sw.Ensemble(sizes) as ens:
        for q, m in enumerate(mem):
            ens.upload(q, *m)
        ens.step(20)
        dts = ens.last_dt()
        for q, (n, _) in enumerate(specs):
            ref = port.run(port.grid(n, n), *mem[q], 20, 0.0)
            assert bitwise_equal(ens.download(q)[0], ref[0])
            assert dts[q] == ref[3][-1]
