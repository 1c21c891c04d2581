"""The C restatement against the golden fixtures made by running the reference
(tests/golden/make_golden.py).  Pins the oracle on any machine."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np
import pytest

from conftest import bitwise_equal

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SMALL = ["random_dry_40x24", "dambreak_trans_48x40", "lake_island_32", "odd_17x33"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def load_case(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    return meta, {k: z[k] for k in z.files if k != "meta"}


@pytest.mark.parametrize("name", SMALL)
def test_port_matches_golden(port, name):
    meta, a = load_case(name)
    p = port.grid(meta["Nx"], meta["Ny"], meta["Lx"], meta["Ly"], cfl=meta["cfl"], bc=meta["bc"])
    h, hu, hv, dts, t, st = port.run(p, a["h"], a["hu"], a["hv"], a["B"], meta["steps"],
                                     meta["dt_fixed"])
    assert st == 0
    assert bitwise_equal(h, a["h_out"]) and bitwise_equal(hu, a["hu_out"])
    assert bitwise_equal(hv, a["hv_out"])
    assert bitwise_equal(dts, a["dts"]) and t == meta["t_end"]


@pytest.mark.parametrize("variant", ["config0_g980665", "config0_g981"])
def test_port_matches_config0_hashes(port, problems, variant):
    """256^2 Gaussian hump, 1000 steps: output SHA-256 equal to the reference's."""
    meta = json.load(open(os.path.join(GOLDEN, "config0_256.json")))[variant]
    N = meta["N"]
    h, hu, hv, B = problems.gauss_hump(N, N)
    if sha(h) != meta["input_sha256"]["h"]:
        pytest.skip("this platform's exp() gives different inputs; fixture inputs not reproducible")
    p = port.grid(N, N, g=meta["g"], cfl=meta["cfl"])
    assert port.stable_dt(p, h, hu, hv) == meta["dt"]
    ho, huo, hvo, _, t, st = port.run(p, h, hu, hv, B, meta["steps"], meta["dt"])
    assert st == 0
    assert sha(ho) == meta["output_sha256"]["h"]
    assert sha(huo) == meta["output_sha256"]["hu"]
    assert sha(hvo) == meta["output_sha256"]["hv"]
    assert t == meta["t_end"]


def test_lake_at_rest_reference_behaviour():
    """Reference behaviour kept as is: with an emerged island, the 1e-8 positivity floor
    breaks the balance at dry cells, so momentum is not exactly zero there."""
    meta, a = load_case("lake_island_32")
    wet = a["h"][2:-2, 2:-2] > 1e-3
    assert (~wet).any()
    assert np.abs(a["hu_out"]).max() > 0.0
