"""x-slab decomposition (shallow-water_gb300/slabs.py; the reference's multi-GPU split,
cuda_solver_4gpu.hpp:281-304): the slabs stepped with per-stage halo exchange and one
global CFL dt give bitwise the whole grid's result.  CPU: slabs computed by the oracle,
in one process and as gloo ranks (world size 2 and 3).  GPU: slabs as library contexts
with x_halo sides on one device, against one context over the whole grid."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

import slab_oracle as so


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def whole_grid(port, Nx, Ny, bc, steps, seed=5):
    h, hu, hv, B = so.case(Nx, Ny, bc, seed)
    p = port.grid(Nx, Ny, bc=so.BC[bc], threads=1)
    oh, ohu, ohv, dts, t, st = port.run(p, h, hu, hv, B, steps)
    assert st == 0
    return (oh, ohu, ohv), t


def test_partition(sw):
    S = sw.slabs
    assert S.partition(10, 3) == [(0, 3), (3, 6), (6, 10)]
    assert S.partition(64, 1) == [(0, 64)]
    with pytest.raises(ValueError):
        S.partition(5, 3)


@pytest.mark.parametrize("bc", ["reflecting", "transmissive"])
@pytest.mark.parametrize("parts", [2, 3, 4])
def test_slabs_in_process_bitwise(sw, port, bc, parts):
    Nx, Ny, steps = 23, 17, 12
    want, t_want = whole_grid(port, Nx, Ny, bc, steps)
    h, hu, hv, B = so.case(Nx, Ny, bc, 5)
    grid = sw.slabs.SlabGrid(Nx, Ny, bc=bc, parts=parts,
                             make_local=so.make_oracle_local(Ny, port.G_REFERENCE, 0.45, bc))
    grid.upload(h, hu, hv, B)
    t = grid.step(steps)
    got = grid.download()
    assert t == t_want
    for a, b in zip(got, want):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("world,bc", [(2, "reflecting"), (3, "transmissive")])
def test_slabs_gloo_ranks_bitwise(port, tmp_path, world, bc):
    import torch.multiprocessing as mp
    Nx, Ny, steps = 20, 12, 8
    mp.spawn(so.gloo_worker, args=(world, free_port(), Nx, Ny, bc, steps, str(tmp_path)),
             nprocs=world, join=True)
    r = np.load(os.path.join(tmp_path, "slabs.npz"))
    want, t_want = whole_grid(port, Nx, Ny, bc, steps)
    assert float(r["t"]) == t_want
    for k, b in zip(("h", "hu", "hv"), want):
        assert np.array_equal(r[k], b)
    # the records rank 0 wrote from the gathered slabs: t = 0 and the end state
    from ncclassic import ClassicFile
    f = ClassicFile(os.path.join(tmp_path, "slabs.nc"))
    assert f.numrecs == 2 and f.read("time").tolist() == [0.0, t_want]
    h0 = so.case(Nx, Ny, bc, 5)[0]
    assert np.array_equal(f.read("h")[0].astype(np.float64), h0[2:-2, 2:-2])
    for k, b in zip(("h", "hu", "hv"), want):
        assert np.array_equal(f.read(k)[1].astype(np.float64), b[2:-2, 2:-2])


@pytest.mark.gpu
@pytest.mark.parametrize("bc", ["reflecting", "transmissive"])
@pytest.mark.parametrize("parts", [2, 3])
def test_slabs_gpu_bitwise(gpu_lib, sw, port, bc, parts):
    Nx, Ny, steps = 70, 45, 15
    h, hu, hv, B = so.case(Nx, Ny, bc, 5)
    with sw.Solver(Nx, Ny, bc=bc) as s:
        s.upload(h, hu, hv, B)
        t_want = s.step(steps)
        want = s.download()
    grid = sw.slabs.SlabGrid(Nx, Ny, bc=bc, parts=parts)
    try:
        grid.upload(h, hu, hv, B)
        t = grid.step(steps)
        got = grid.download()
    finally:
        grid.close()
    assert t == t_want
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
    oracle, t_o = whole_grid(port, Nx, Ny, bc, steps)
    for a, b in zip(got, oracle):
        assert np.array_equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("bc", ["reflecting", "transmissive"])
@pytest.mark.parametrize("parts", [2, 3, 4])
def test_device_slabs_bitwise(gpu_lib, sw, port, bc, parts):
    """The single-process slab group (device-side exchange overlapped with each stage's
    inner tile rows, device-side max-speed gather) on one GPU: bitwise one context and
    the oracle, adaptive dt over several calls; slabs of one and two tile rows included."""
    Nx, Ny, steps = 70, 45, 15
    h, hu, hv, B = so.case(Nx, Ny, bc, 5)
    with sw.Solver(Nx, Ny, bc=bc) as s:
        s.upload(h, hu, hv, B)
        t_want = s.step(steps)
        want = s.download()
    with sw.slabs.DeviceSlabGrid(Nx, Ny, bc=bc, parts=parts) as grid:
        grid.upload(h, hu, hv, B)
        grid.step(4)
        t = grid.step(steps - 4)
        got = grid.download()
    assert t == t_want
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
    oracle, t_o = whole_grid(port, Nx, Ny, bc, steps)
    for a, b in zip(got, oracle):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_device_slabs_large_fixed_dt_and_thin_slabs(gpu_lib, sw, problems):
    """A dam break over seeded bathymetry (TMA interior tiles, inner and edge launches of
    several tile rows) and a grid whose slabs are 2-3 rows thick, with fixed dt."""
    B, _ = problems.gaussian_sum_bathymetry(520, 300, n=16, seed=3, bc="transmissive")
    h, hu, hv = problems.dam_break(B)
    for Nx, parts in ((520, 3), (11, 4)):
        Bs = np.ascontiguousarray(B[:Nx + 4])
        hs, hus, hvs = (np.ascontiguousarray(a[:Nx + 4]) for a in (h, hu, hv))
        with sw.Solver(Nx, 300, bc="transmissive") as s:
            s.upload(hs, hus, hvs, Bs)
            dt = 0.5 * s.stable_dt()
            t_want = s.step(12, dt)
            want = s.download()
        with sw.slabs.DeviceSlabGrid(Nx, 300, bc="transmissive", parts=parts) as grid:
            grid.upload(hs, hus, hvs, Bs)
            t = grid.step(12, dt)
            got = grid.download()
        assert t == t_want
        for a, b in zip(got, want):
            assert np.array_equal(a, b), (Nx, parts)
