"""One grid split into x-slabs, one per GPU (or several on one GPU).

The reference's 4-GPU backend splits the rows i (x, the slow index) into contiguous
slabs (build_subdomains, cuda_solver_4gpu.hpp:281-304) and, after every RK stage,
exchanges the two ghost rows each slab needs from each neighbour.  Here every slab is a
``Solver`` created with ``x_halo`` set on its interface sides, so its stage kernels read
those ghost rows as stored.  One step is

    dt = cfl * min(dx, dy) / max over all slabs of the max wave speed of U^n
    for s in 1, 2, 3:  every slab runs stage s (swe_stage) with that dt, then the buffer
                       stage s wrote (s % 3) exchanges its interface rows,

which is bitwise the step of the whole grid: every interface flux sees the same stencil
values, and the global max speed is an exact max.  The exchange is the only
communication besides one max-reduction of the speed per step.

Two drivers:

- :class:`DeviceSlabGrid` (one process, one or several GPUs; the reference's 4-GPU
  model): the library's ``swe_slabs_*``, which keeps the exchange and the max-reduction
  on the devices (peer copies overlapped with each stage's inner tile rows, events
  between the slabs' streams, no host round trip per step).
- :class:`SlabGrid`: one slab per process (``comm``, a torch.distributed group) or
  every slab here (``comm=None``), stepped stage by stage through ``swe_stage`` with the
  interface rows passed through host arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from .solver import Solver, SweError, _BC, _dp, _ghosted


def partition(Nx: int, parts: int):
    """Row ranges [r0, r1) of `parts` slabs whose sizes differ by at most one."""
    if parts < 1 or Nx < 2 * parts:
        raise ValueError(f"cannot split {Nx} rows into {parts} slabs of at least 2 rows")
    return [(k * Nx // parts, (k + 1) * Nx // parts) for k in range(parts)]


class TorchComm:
    """The ranks of a torch.distributed group: gloo for host arrays, NCCL for a GPU
    device (the arrays then travel as CUDA tensors)."""

    def __init__(self, group=None, device=None):
        import torch
        import torch.distributed as dist
        self.torch, self.dist, self.group = torch, dist, group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)
        self.device = device or "cpu"

    def _peer(self, r):
        return r if self.group is None else self.dist.get_global_rank(self.group, r)

    def allreduce_max(self, x: float) -> float:
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX, group=self.group)
        return float(t.item())

    def exchange(self, sends: dict, shape) -> dict:
        """Sends sends[r] to rank r and returns {r: array received from r}."""
        torch = self.torch
        reqs, recv = [], {}
        for r in sorted(sends):
            recv[r] = torch.empty(shape, dtype=torch.float64, device=self.device)
            reqs.append(self.dist.irecv(recv[r], src=self._peer(r), group=self.group))
        for r in sorted(sends):
            t = torch.as_tensor(np.ascontiguousarray(sends[r])).to(self.device)
            reqs.append(self.dist.isend(t, dst=self._peer(r), group=self.group))
        for q in reqs:
            q.wait()
        return {r: v.cpu().numpy() for r, v in recv.items()}

    def all_gather(self, obj):
        out = [None] * self.size
        self.dist.all_gather_object(out, obj, group=self.group)
        return out


class SlabGrid:
    """A (Nx, Ny) grid stepped as x-slabs.

    comm None: all `parts` slabs in this process.  comm a TorchComm: `comm.size` slabs,
    this process holding slab `comm.rank`.  `make_local(rows, dx, dy, halo_lo, halo_hi)`
    builds one slab's solver with the grid's cell sizes (default: a GPU ``Solver`` on
    `device`); anything with upload / download / stage / halo_pack / halo_unpack /
    max_wave_speed works."""

    def __init__(self, Nx: int, Ny: int, Lx: float = 1.0, Ly: float = 1.0,
                 g: float = 9.80665, cfl: float = 0.45, bc="reflecting", parts: int = 2,
                 comm: TorchComm | None = None, device: int = 0, make_local=None):
        self.Nx, self.Ny, self.comm = Nx, Ny, comm
        self.parts = comm.size if comm is not None else parts
        self.ranges = partition(Nx, self.parts)
        self.dx, self.dy = Lx / Nx, Ly / Ny
        self.cfl_min_dxdy = cfl * min(self.dx, self.dy)  # compute_stable_dt numerator
        self.mine = [comm.rank] if comm is not None else list(range(self.parts))
        if make_local is None:
            def make_local(rows, dx, dy, lo, hi):
                return Solver(rows, Ny, dx * rows, Ly, g, cfl, bc, "fp64", device,
                              x_halo=(lo, hi), dx=dx, dy=dy)
        self.local = {}
        for k in self.mine:
            r0, r1 = self.ranges[k]
            self.local[k] = make_local(r1 - r0, self.dx, self.dy, k > 0, k < self.parts - 1)
        self.time = 0.0

    def close(self):
        for s in self.local.values():
            if hasattr(s, "close"):
                s.close()

    def upload(self, h, hu, hv, B):
        """Full ghosted (Nx + 4, Ny + 4) arrays; each slab takes its rows plus two on
        either side (its neighbours' rows or the grid's ghosts)."""
        for k, s in self.local.items():
            r0, r1 = self.ranges[k]
            s.upload(*(np.ascontiguousarray(a[r0:r1 + 4]) for a in (h, hu, hv, B)))
        self.time = 0.0

    def _exchange(self, buffer: int):
        """Interface rows of `buffer` to each neighbour's ghost rows."""
        out = {}  # (to slab, its side) -> rows
        for k, s in self.local.items():
            if k > 0:
                out[(k - 1, 1)] = s.halo_pack(buffer, 0)
            if k < self.parts - 1:
                out[(k + 1, 0)] = s.halo_pack(buffer, 1)
        remote = {key: v for key, v in out.items() if key[0] not in self.local}
        for (k, side), rows in out.items():
            if k in self.local:
                self.local[k].halo_unpack(buffer, side, rows)
        if self.comm is not None:
            me = self.comm.rank
            sends = {k: rows for (k, _), rows in remote.items()}
            got = self.comm.exchange(sends, (3, 2, self.Ny + 4))
            for r, rows in got.items():
                self.local[me].halo_unpack(buffer, 0 if r < me else 1, rows)

    def stable_dt(self) -> float:
        ms = max(s.max_wave_speed() for s in self.local.values())
        if self.comm is not None:
            ms = self.comm.allreduce_max(ms)
        return 1.0e100 if ms <= 1.0e-8 else self.cfl_min_dxdy / ms  # HPC_kernels.hpp:296-297

    def step(self, n_steps: int = 1, dt: float | None = None) -> float:
        """n_steps RK3 steps; dt None = adaptive CFL dt of the whole grid per step."""
        for _ in range(n_steps):
            d = dt if dt else self.stable_dt()
            for st in (1, 2, 3):
                for s in self.local.values():
                    s.stage(st, d)
                self._exchange(st % 3)
            self.time += d
        return self.time

    def write_snapshot(self, writer, **metadata):
        """Appends the whole grid's state to an ``output.NetCDFWriter`` (one record at
        ``self.time``).  The slabs are gathered first, as the reference's 4-GPU solver
        gathers to one host before writing; with ranks, the rank holding slab 0 writes
        and the others pass ``writer=None``."""
        state = self.download()
        if self.comm is None or self.comm.rank == 0:
            writer.write_snapshot(state, self.time, **metadata)

    def download(self):
        """The whole grid's (h, hu, hv), ghosts by the wall rule, on every process."""
        pieces = {k: s.download() for k, s in self.local.items()}
        if self.comm is not None:
            allp = self.comm.all_gather(pieces)
            pieces = {k: v for d in allp for k, v in d.items()}
        out = tuple(np.empty((self.Nx + 4, self.Ny + 4)) for _ in range(3))
        for k, arrs in pieces.items():
            r0, r1 = self.ranges[k]
            for f in range(3):
                lo = 0 if k == 0 else 2
                hi = r1 - r0 + (4 if k == self.parts - 1 else 2)
                out[f][r0 + lo:r0 + hi] = arrs[f][lo:hi]
        return out


class DeviceSlabGrid:
    """A (Nx, Ny) grid as ``parts`` x-slabs of this process on ``devices`` (one per slab;
    default all on ``device``), stepped by the library with device-side exchange."""

    def __init__(self, Nx: int, Ny: int, Lx: float = 1.0, Ly: float = 1.0,
                 g: float = 9.80665, cfl: float = 0.45, bc="reflecting", parts: int = 2,
                 devices=None, device: int = 0):
        self._lib = L.lib()
        p = L.SweParams()
        self._lib.swe_params_default(ctypes.byref(p))
        p.Nx, p.Ny, p.Lx, p.Ly, p.g, p.cfl = Nx, Ny, Lx, Ly, g, cfl
        p.bc = _BC[bc] if isinstance(bc, str) else int(bc)
        p.device = device
        self.Nx, self.Ny, self.parts = Nx, Ny, parts
        devs = None
        if devices is not None:
            devs = (ctypes.c_int * parts)(*[int(d) for d in devices])
        self._ctx = ctypes.c_void_p()
        st = self._lib.swe_slabs_create(ctypes.byref(p), parts, devs, ctypes.byref(self._ctx))
        if st != L.SWE_OK:
            self._ctx = ctypes.c_void_p()
            raise SweError(st, "swe_slabs_create: " + self._lib.swe_status_string(st).decode())
        self.time = 0.0

    def _check(self, st, what):
        if st != L.SWE_OK:
            msg = self._lib.swe_slabs_last_error(self._ctx).decode() if self._ctx else ""
            raise SweError(st, f"{what}: {self._lib.swe_status_string(st).decode()}: {msg}")

    def close(self):
        if self._ctx:
            self._lib.swe_slabs_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def upload(self, h, hu, hv, B):
        arrs = [_ghosted(a, self.Nx, self.Ny, n) for a, n in ((h, "h"), (hu, "hu"), (hv, "hv"), (B, "B"))]
        self._check(self._lib.swe_slabs_upload(self._ctx, *(_dp(a) for a in arrs)), "swe_slabs_upload")
        self.time = 0.0

    def download(self):
        out = tuple(np.empty((self.Nx + 4, self.Ny + 4)) for _ in range(3))
        self._check(self._lib.swe_slabs_download(self._ctx, *(_dp(a) for a in out)),
                    "swe_slabs_download")
        return out

    def step(self, n_steps: int = 1, dt: float | None = None) -> float:
        t = ctypes.c_double(self.time)
        st = self._lib.swe_slabs_step(self._ctx, int(n_steps), float(dt or 0.0), ctypes.byref(t))
        self.time = t.value
        self._check(st, "swe_slabs_step")
        return self.time

    def last_step_ms(self) -> float:
        v = ctypes.c_double()
        self._check(self._lib.swe_slabs_last_step_ms(self._ctx, ctypes.byref(v)),
                    "swe_slabs_last_step_ms")
        return v.value

    def kernel_launches(self) -> int:
        return int(self._lib.swe_slabs_kernel_launches(self._ctx))
