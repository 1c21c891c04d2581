"""The integer-pipe FP64 helpers of the FP64 kernel are bitwise equal to the plain IEEE
expressions they replace (CPU build of the same header; edge values, random operands
and constructed rounding ties)."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from conftest import ROOT


@pytest.mark.skipif(not shutil.which("g++"), reason="g++ not available")
def test_exact_helpers_bitwise(tmp_path):
    exe = tmp_path / "exact_check"
    src = os.path.join(ROOT, "tests", "cpp", "exact_helpers_check.cpp")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-o", str(exe), src],
                   check=True)
    r = subprocess.run([str(exe), "1000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "0 mismatches" in r.stdout


def _finite_doubles(rng, n, lo=-300, hi=300):
    """Random finite doubles over a wide exponent range, with zeros and subnormals."""
    import numpy as np
    m = rng.uniform(1.0, 2.0, n) * rng.choice([-1.0, 1.0], n)
    x = np.ldexp(m, rng.integers(lo, hi, n))
    x[rng.random(n) < 0.02] = 0.0
    sub = rng.random(n) < 0.02
    x[sub] = np.ldexp(rng.uniform(0.0, 1.0, int(sub.sum())), -1030)
    return x


def test_one_division_wave_speed_identity():
    """The stage-3 wave speed max(|hu|, |hv|) / h + c equals the reference's
    max(|hu| / h + c, |hv| / h + c) bitwise for finite values: correctly rounded
    division and addition are monotonic.  Checked in numpy's IEEE binary64 on random
    and near-tied operands."""
    import numpy as np
    rng = np.random.default_rng(7)
    n = 400_000
    h = np.abs(_finite_doubles(rng, n, -40, 10)) + 1e-8
    hu = _finite_doubles(rng, n, -60, 20)
    hv = _finite_doubles(rng, n, -60, 20)
    # near ties: |hv| within a few ulps of |hu|
    k = n // 4
    hv[:k] = np.nextafter(hu[:k], np.inf * np.sign(hu[:k] + 0.5))
    c = np.sqrt(9.80665 * h)
    with np.errstate(over="ignore"):
        ref = np.maximum(np.abs(hu) / h + c, np.abs(hv) / h + c)
        new = np.maximum(np.abs(hu), np.abs(hv)) / h + c
    fin = np.isfinite(ref)
    assert fin.mean() > 0.99
    assert np.array_equal(ref[fin].view(np.uint64), new[fin].view(np.uint64))
