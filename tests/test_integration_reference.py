"""The GB300 backend inside the reference's own SolverAssembly.

Copies the reference tree, adds the GB300 backend with
shallow-water_gb300/integration.py, compiles the reference app (apps/main.cpp, its
config parser and sanity checks) with include/swe_gb300_solver.hpp against
libswe_gb300.so, and runs it on simulation_config.toml files.  Runs where the
reference sources and g++ are available (CPU: without a GPU the backend must fail
with the library's no-device error, after the config parsed and dispatched)."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from conftest import ROOT
from oracle.ref import reference_dir

REF = reference_dir()
pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(REF) or not shutil.which("g++"),
                                reason="reference sources or g++ not available")

CONFIG = """[mesh]
Lx = 1.0
Ly = 1.0
nG = 2
Nx = 32
Ny = 32
spatial_unit_x = "m"
spatial_unit_y = "m"
spatial_unit_h = "m"

[bathymetry]
type = "GaussHill"
b0 = 0.0
bathy_x0 = 0.5
bathy_y0 = 0.5
bathy_sigma_x = 0.1
bathy_sigma_y = 0.1
bathy_peak_height = 0.3

[boundary]
type = "ReflectingWalls"

[initial_condition]
type = "GaussInitial"
h0 = 1.0
peak_height = 0.1
x0 = 0.5
y0 = 0.5
sigma_x = 0.07
sigma_y = 0.07
dam_height = 2.0
dam_x = 0.5
dam_x0 = 0.5
dam_y0 = 0.5
dam_radius = 0.2

[solver]
reconstruction = "MUSCL"
riemann = "HLL"
time = "SSPRK3"

[time]
end_time = 0.02
time_steps = 40
cfl = 0.45
time_unit = "s"
save_every = 10

[backend]
type = "{backend}"
threads = 1

[output]
compute_eta = false
path = "output/simulation.nc"
"""


def build_app(tree, name, extra=()):
    libdir = os.path.join(ROOT, "shallow-water_gb300")
    exe = tree / name
    cmd = ["g++", "-std=c++17", "-O1", "-DUSE_OPENMP=0", "-DUSE_CUDA=0", "-DUSE_CUDA_4=0",
           "-DUSE_GB300=1", *extra, "-include", "iostream", f"-I{tree}", f"-I{ROOT}/include",
           f"-I{ROOT}/oracle/ref/stub", "-w",
           str(tree / "apps/main.cpp"), str(tree / "configs/simulation_config.cpp"),
           str(tree / "tests/sanity_checks/sanity_checks.cpp"),
           os.path.join(ROOT, "oracle/ref/netcdf_noop.cpp"),
           f"-L{libdir}", "-lswe_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.fixture(scope="module")
def patched_tree(tmp_path_factory, sw):
    from importlib import import_module
    integ = import_module("shallow-water_gb300.integration")
    tree = tmp_path_factory.mktemp("ref") / "shallow-water"
    shutil.copytree(REF, tree, ignore=shutil.ignore_patterns("docs", "python", ".git"))
    integ.patch_reference_tree(str(tree))
    return tree


@pytest.fixture(scope="module")
def patched_app(patched_tree):
    return patched_tree, build_app(patched_tree, "swe_solver_gb300")


def run_app(tree, exe, backend):
    cfg = tree / "configs" / "simulation_config.toml"
    os.chmod(cfg, 0o644)
    cfg.write_text(CONFIG.replace("{backend}", backend))
    return subprocess.run([str(exe)], cwd=tree, capture_output=True, text=True, timeout=120)


def test_patch_touches_every_site(patched_app):
    tree, _ = patched_app
    assert "GB300 };" in (tree / "configs/config.hpp").read_text()
    assert '"GB300") return BackendType::GB300' in (tree / "configs/simulation_config.cpp").read_text()
    assert 'return "GB300";' in (tree / "configs/parse_config_helper.hpp").read_text()
    sa = (tree / "include/solver_assembly/solver_assembly.hpp").read_text()
    assert "FastHLLMUSCLBathyGB300Solver solver(cfg_);" in sa
    assert "ENABLE_GB300" in (tree / "CMakeLists.txt").read_text()


def test_unknown_backend_is_rejected_by_the_reference_parser(patched_app):
    tree, exe = patched_app
    r = run_app(tree, exe, "GB3000")
    assert r.returncode != 0
    assert "Unknown backend type: GB3000" in r.stderr


def test_gb300_backend_dispatches(patched_app):
    tree, exe = patched_app
    r = run_app(tree, exe, "GB300")
    import torch
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stderr
        assert "GB300 fused-stage solver active" in r.stdout
    else:
        assert r.returncode != 0
        assert "GB300 backend: swe_create: no CUDA device" in r.stderr


def test_gb300_backend_with_native_output(patched_tree):
    """The class built with SWE_GB300_NATIVE_OUTPUT=1 (snapshots through the library's
    own NetCDF writer) compiles and dispatches the same way."""
    exe = build_app(patched_tree, "swe_solver_gb300_native", ["-DSWE_GB300_NATIVE_OUTPUT=1"])
    r = run_app(patched_tree, exe, "GB300")
    import torch
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stderr
        out = patched_tree / "output" / "simulation.nc"
        assert out.exists() and out.read_bytes()[:4] == b"CDF\x02"
    else:
        assert r.returncode != 0
        assert "GB300 backend: swe_create: no CUDA device" in r.stderr


def test_gb300_backend_dispatches_modular_combinations(patched_app):
    """[solver] PiecewiseConst + Rusanov over no bathymetry (a Serial-backend combination)
    reaches the GB300 class, which runs it with the modular scheme."""
    tree, exe = patched_app
    cfg = tree / "configs" / "simulation_config.toml"
    os.chmod(cfg, 0o644)
    text = CONFIG.replace("{backend}", "GB300").replace('reconstruction = "MUSCL"',
                                                          'reconstruction = "PiecewiseConst"')
    text = text.replace('riemann = "HLL"', 'riemann = "Rusanov"').replace('type = "GaussHill"',
                                                                        'type = "None"')
    cfg.write_text(text)
    r = subprocess.run([str(exe)], cwd=tree, capture_output=True, text=True, timeout=120)
    import torch
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stderr
        assert "GB300 modular solver active (PiecewiseConst + Rusanov)" in r.stdout
    else:
        assert r.returncode != 0
        assert "Unsupported" not in r.stderr
        assert "GB300 backend: swe_create: no CUDA device" in r.stderr
