"""Test helpers for the slab decomposition: a slab whose compute is the CPU oracle
(oracle/port.py), so the host logic of shallow-water_gb300/slabs.py (partition, halo
rows, exchange order, global dt) runs and is checked on machines without a GPU, and a
world-size-N gloo worker."""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import port  # noqa: E402

BC = {"reflecting": port.BC_REFLECTING, "transmissive": port.BC_TRANSMISSIVE}


class OracleSlab:
    """One slab on the oracle: buffers U^n, U^(1), U^(2) as ghosted numpy arrays."""

    def __init__(self, rows, Ny, dx, dy, g, cfl, bc):
        self.rows = rows
        self.p = port.grid(rows, Ny, dx * rows, dy * Ny, g, cfl, BC[bc], threads=1, dx=dx, dy=dy)
        self.buf = [None, None, None]

    def upload(self, h, hu, hv, B):
        self.buf[0] = [np.array(a, dtype=np.float64) for a in (h, hu, hv)]
        self.B = np.array(B, dtype=np.float64)

    def stage(self, st, dt):
        src = self.buf[0] if st == 1 else self.buf[st - 1]
        h, hu, hv, status = port.stage(self.p, st, dt, self.buf[0], src, self.B)
        assert status == 0
        self.buf[st % 3] = [h, hu, hv]

    def halo_pack(self, b, side):
        r = 2 if side == 0 else self.rows
        return np.stack([a[r:r + 2].copy() for a in self.buf[b]])

    def halo_unpack(self, b, side, rows):
        r = 0 if side == 0 else self.rows + 2
        for f in range(3):
            self.buf[b][f][r:r + 2] = rows[f]

    def max_wave_speed(self):
        return port.max_wave_speed(self.p, *self.buf[0])

    def download(self):
        return tuple(a.copy() for a in self.buf[0])


def make_oracle_local(Ny, g, cfl, bc):
    def make(rows, dx, dy, lo, hi):
        return OracleSlab(rows, Ny, dx, dy, g, cfl, bc)
    return make


def case(Nx, Ny, bc, seed):
    """A dam break with a noisy momentum over seeded bathymetry; ghosts of every field
    by the wall rule, as the whole grid has them before its first stage."""
    P = importlib.import_module("shallow-water_gb300.problems")
    rng = np.random.default_rng(seed)
    B, _ = P.gaussian_sum_bathymetry(Nx, Ny, n=6, rng=rng, bc=bc)
    h, hu, hv = P.dam_break(B)
    hu = np.ascontiguousarray(hu + 0.01 * rng.standard_normal(hu.shape))
    port.fill_ghosts(port.grid(Nx, Ny, bc=BC[bc]), h, hu, hv)
    return h, hu, hv, B


def gloo_worker(rank, world, port_no, Nx, Ny, bc, steps, out_dir):
    """One rank of a gloo group stepping its slab on the oracle; rank 0 saves the
    assembled grid and the time."""
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port_no)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        slabs = importlib.import_module("shallow-water_gb300.slabs")
        h, hu, hv, B = case(Nx, Ny, bc, seed=5)
        grid = slabs.SlabGrid(Nx, Ny, bc=bc, comm=slabs.TorchComm(),
                              make_local=make_oracle_local(Ny, port.G_REFERENCE, 0.45, bc))
        grid.upload(h, hu, hv, B)
        writer = None
        if rank == 0:  # the gathered grid as NetCDF records, written by rank 0 alone
            out_mod = importlib.import_module("shallow-water_gb300.output")
            writer = out_mod.NetCDFWriter(os.path.join(out_dir, "slabs.nc"), (Nx, Ny, 1.0, 1.0))
            writer.write_bathymetry(B)
        grid.write_snapshot(writer, dt=0.0, backend="GB300")
        t = grid.step(steps)
        grid.write_snapshot(writer)
        out = grid.download()
        if rank == 0:
            writer.close()
            np.savez(os.path.join(out_dir, "slabs.npz"), h=out[0], hu=out[1], hv=out[2], t=t)
        dist.barrier()
    finally:
        dist.destroy_process_group()
