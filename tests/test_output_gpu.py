"""Device snapshots (swe_snapshot_write): records packed on the GPU and written by the
writer thread while the solver keeps stepping must equal, bit for bit, the state
swe_download returns at the same step, and (FP64) the oracle's state."""
from __future__ import annotations

import numpy as np
import pytest

from ncclassic import ClassicFile

pytestmark = pytest.mark.gpu


def interior(a):
    return np.asarray(a)[2:-2, 2:-2]


def same_bits(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def run_and_record(sw, s, w, schedule, dt):
    """Steps `s` by each n in schedule, writing a device record after each (and at t=0);
    returns the downloads taken right after each write."""
    want = []
    w.write_snapshot(s, s.time)
    want.append((s.time, *s.download()))
    for n in schedule:
        s.step(n, dt)
        w.write_snapshot(s, s.time)  # async; the next step queues behind the pack only
        want.append((s.time, *s.download()))
    w.flush()
    return want


def check_file(path, want, fmt=2):
    f = ClassicFile(path)
    assert f.version == fmt and f.numrecs == len(want)
    t = f.read("time")
    for k, (tk, h, hu, hv) in enumerate(want):
        assert t[k] == tk
        for name, a in (("h", h), ("hu", hu), ("hv", hv)):
            got = f.read(name)[k].astype(np.float64)
            assert same_bits(got, interior(a)), (name, k)


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_device_records_equal_downloads(gpu_lib, sw, problems, tmp_path, precision):
    Nx, Ny = 96, 80
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=21)
    path = str(tmp_path / f"dev_{precision}.nc")
    with sw.Solver(Nx, Ny, Lx=1.5, Ly=1.0, precision=precision) as s:
        s.upload(h, hu, hv, B)
        w = sw.output.NetCDFWriter(path, s, "m", "m", "m", "s", save_every=1)
        w.write_bathymetry(B)
        # back-to-back records (1-step gaps) exercise the wait on a busy staging buffer
        want = run_and_record(sw, s, w, [1, 1, 1, 4, 2], 0.0)
        copy_s, write_s, nbytes = w.stats()
        w.close()
    assert nbytes == len(want) * 3 * Nx * Ny * 8
    check_file(path, want)
    f = ClassicFile(path)
    assert same_bits(f.read("B").astype(np.float64), interior(B))


def test_device_records_chunked_and_mixed_with_host(gpu_lib, sw, problems, tmp_path):
    """2048^2: a record's 100 MB leave the staging buffer in two 64 MB chunks, the first
    ending inside hu; host records interleave in order with device records."""
    N = 2048
    h, hu, hv, B = problems.random_state(N, N, seed=5)
    path = str(tmp_path / "big.nc")
    with sw.Solver(N, N) as s:
        s.upload(h, hu, hv, B)
        w = sw.output.NetCDFWriter(path, s, save_every=2)
        w.write_bathymetry(B)
        want = []
        w.write_snapshot(s, s.time)
        want.append((s.time, *s.download()))
        s.step(2)
        host = s.download()
        w.write_snapshot(host, s.time)  # host record after the pending device record
        want.append((s.time, *host))
        s.step(2)
        w.write_snapshot(s, s.time)
        want.append((s.time, *s.download()))
        w.close()
    check_file(path, want)


def test_device_record_equals_oracle(gpu_lib, sw, port, problems, tmp_path):
    Nx, Ny, steps, dt = 64, 72, 12, 2.0e-3
    h, hu, hv, B = (np.array(a, dtype=np.float64) for a in problems.random_state(Nx, Ny, seed=8))
    p = port.grid(Nx, Ny)
    port.fill_ghosts(p, h, hu, hv)
    oh, ohu, ohv, _, ot, st = port.run(p, h, hu, hv, B, steps, dt)
    assert st == 0
    path = str(tmp_path / "oracle.nc")
    with sw.Solver(Nx, Ny) as s:
        s.upload(h, hu, hv, B)
        w = sw.output.NetCDFWriter(path, s)
        s.step(steps, dt)
        w.write_snapshot(s, s.time)
        w.close()
    f = ClassicFile(path)
    for name, a in (("h", oh), ("hu", ohu), ("hv", ohv)):
        assert same_bits(f.read(name)[0].astype(np.float64), interior(a)), name
    assert f.read("time")[0] == ot


def test_run_with_writer(gpu_lib, sw, problems, tmp_path):
    """Solver.run(writer=...): a record at t = 0, every save_every steps and at the end,
    equal to the on_snapshot downloads; the run metadata on the file."""
    Nx, Ny = 48, 40
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=3)
    path = str(tmp_path / "run.nc")
    seen = []
    with sw.Solver(Nx, Ny) as s:
        s.upload(h, hu, hv, B)
        w = sw.output.NetCDFWriter(path, s, save_every=4)
        w.write_bathymetry(B)
        s.run(0.02, 10, save_every=4, on_snapshot=lambda k, t, *U: seen.append((t, *U)),
              writer=w, bathymetry_name="random")
        w.close()
    assert len(seen) == 4  # t = 0, steps 4, 8 and the final 10
    check_file(path, seen)
    f = ClassicFile(path)
    assert f.gatts["backend"] == "GB300" and f.gatts["bathymetry"] == "random"
    assert f.gatts["dt"].item() == 0.02 / 10
