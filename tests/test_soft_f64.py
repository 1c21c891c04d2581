"""The integer-pipe binary64 division and square root used by the FP64 kernels are
bitwise equal to IEEE round-to-nearest division and square root: on the CPU against the
host's operations (also with the FP32 seeds perturbed far beyond the hardware
approximations' error), and on the GPU against the device's own operations."""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


@pytest.mark.skipif(not shutil.which("g++"), reason="g++ not available")
@pytest.mark.parametrize("hook", [False, True], ids=["seeds", "perturbed-seeds"])
def test_soft_div_sqrt_bitwise_cpu(tmp_path, hook):
    exe = tmp_path / "soft_check"
    src = os.path.join(ROOT, "tests", "cpp", "soft_f64_check.cpp")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-o", str(exe), src]
    if hook:
        cmd.insert(1, "-DSWE_SOFT_SEED_HOOK")
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe), "400000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    assert " 0 mismatches" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 0xC0FFEE])
def test_soft_div_sqrt_bitwise_gpu(gpu_lib, seed):
    bad = ctypes.c_longlong(-1)
    st = gpu_lib.swe_selftest_soft_f64(1 << 24, seed, ctypes.byref(bad))
    assert st == 0
    assert bad.value == 0
