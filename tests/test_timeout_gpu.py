"""The stage kernels' bounded TMA waits end a whole launch, not just a tile, and leave the
context usable, tested without a GPU fault.

- The give-up path itself: blocks arm a transaction barrier for bytes that no copy
  delivers and wait on it through the stage kernels' own helpers (no copy is issued, so
  nothing is left in flight).  The waits give up, the launch reports SWE_ERR_TIMEOUT, and
  only the blocks resident at the start waited: every later block returned at its flag
  check, so the launch took about two deadlines, not one per wave of blocks.
- The per-launch exit of the real stage kernels: the host starts a call with the timeout
  bit already set in the context's flag word (a flag the kernels would set after a failed
  wait).  Every tile then returns before staging anything, the call returns
  SWE_ERR_TIMEOUT at once, and the next upload and steps give the oracle's results.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import bitwise_equal

pytestmark = pytest.mark.gpu

SWE_ERR_TIMEOUT = 5


def dam_break(problems, nx, ny, seed):
    B, _ = problems.gaussian_sum_bathymetry(nx, ny, seed=seed, bc="transmissive")
    return (*problems.dam_break(B), B)


def test_wait_gives_up_once_per_launch(gpu_lib, sw, port, problems):
    ctas, deadline_ms = 100_000, 2.0
    waited, ms = ctypes.c_longlong(-1), ctypes.c_double(-1.0)
    st = gpu_lib.swe_selftest_wait_timeout(ctas, deadline_ms, ctypes.byref(waited),
                                           ctypes.byref(ms))
    assert st == SWE_ERR_TIMEOUT
    # Only the first resident blocks waited (at most 32 per SM on 152 SMs); waiting one
    # wave after another would have taken over 20 waves x 2 deadlines.
    assert 0 < waited.value <= 152 * 32, waited.value
    assert ms.value < 25 * deadline_ms, ms.value
    # The device is still usable: a solver run equals the oracle bitwise.
    h, hu, hv, B = problems.random_state(40, 56, seed=9, q_scale=0.1, b_scale=0.05)
    ref = port.run(port.grid(40, 56, cfl=0.3), h, hu, hv, B, 6, 0.0)
    with sw.Solver(40, 56, cfl=0.3) as s:
        s.upload(h, hu, hv, B)
        s.step(6)
        out = s.download()
    for k in range(3):
        assert bitwise_equal(out[k], ref[k])


@pytest.mark.parametrize("path", ["step", "step_host", "stage"])
def test_preset_timeout_ends_the_call_and_context_recovers(gpu_lib, sw, port, problems, path):
    N, M = 256, 192  # interior tiles, so the TMA path runs
    h, hu, hv, B = dam_break(problems, N, M, seed=4)
    ref = port.run(port.grid(N, M, cfl=0.45, bc=port.BC_TRANSMISSIVE), h, hu, hv, B, 5, 0.0)
    with sw.Solver(N, M, bc="transmissive") as s:
        s.upload(h, hu, hv, B)
        assert gpu_lib.swe_test_preset_timeout(s._ctx) == 0
        with pytest.raises(sw.SweError) as ei:
            if path == "step":
                s.step(20)
            elif path == "step_host":
                s.step_host(h, hu, hv, B, n_steps=3)
            else:
                s.stage(1, 1e-4)
        assert ei.value.status == SWE_ERR_TIMEOUT
        if path == "step":
            assert s.last_step_ms() < 50.0  # 60 launches whose CTAs all returned at once
        s.time = 0.0
        s.upload(h, hu, hv, B)
        s.step(5)
        out = s.download()
    for k in range(3):
        assert bitwise_equal(out[k], ref[k])


def test_preset_timeout_fp32_form(gpu_lib, sw, problems):
    N = 256
    h, hu, hv, B = dam_break(problems, N, N, seed=6)
    with sw.Solver(N, N, bc="transmissive", precision="fp32_mixed") as a, \
            sw.Solver(N, N, bc="transmissive", precision="fp32_mixed") as b:
        a.upload(h, hu, hv, B)
        assert gpu_lib.swe_test_preset_timeout(a._ctx) == 0
        with pytest.raises(sw.SweError) as ei:
            a.step(10)
        assert ei.value.status == SWE_ERR_TIMEOUT
        a.upload(h, hu, hv, B)
        a.step(7)
        b.upload(h, hu, hv, B)
        b.step(7)
        oa, ob = a.download(), b.download()
    for k in range(3):
        assert bitwise_equal(oa[k], ob[k])


@pytest.mark.parametrize("precision", ["fp32_mixed", "fp64"])
def test_preset_timeout_persistent_ensemble(gpu_lib, sw, problems, precision):
    sizes = [(256, 256), (64, 96), (130, 200), (40, 40)]
    mem = [problems.random_state(nx, ny, seed=20 + q, q_scale=0.1, b_scale=0.05)
           for q, (nx, ny) in enumerate(sizes)]
    with sw.Ensemble(sizes, cfl=0.3, precision=precision) as ens, \
            sw.Ensemble(sizes, cfl=0.3, precision=precision) as ref:
        for e in (ens, ref):
            e.set_schedule("8x32", 304)  # persistent: fewer CTAs than tiles
            for q, m in enumerate(mem):
                e.upload(q, *m)
        assert gpu_lib.swe_ens_test_preset_timeout(ens._ctx) == 0
        with pytest.raises(sw.SweError) as ei:
            ens.step(10)
        assert ei.value.status == SWE_ERR_TIMEOUT
        assert ens.last_step_ms() < 50.0
        for q, m in enumerate(mem):
            ens.upload(q, *m)
        ens.step(6)
        ref.step(6)
        for q in range(len(sizes)):
            a, b = ens.download(q), ref.download(q)
            for k in range(3):
                assert bitwise_equal(a[k], b[k]), (q, k)
        assert np.array_equal(ens.times(), ref.times())
