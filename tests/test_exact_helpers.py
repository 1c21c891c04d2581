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
