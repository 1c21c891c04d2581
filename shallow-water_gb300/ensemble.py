"""Host side of the batched-ensemble C ABI (swe_ens_* in include/swe_gb300.h).

An :class:`Ensemble` holds many independent grids of uneven sizes on one GPU and
advances all of them with one launch per RK stage (per-instance CFL dt), replaying
whole RK3 steps from CUDA graphs.  :meth:`Ensemble.tune` runs the library's autotuner
(tile shape x CTA count) and can cache the choice in a JSON file keyed by the
ensemble's signature, so later runs of the same configuration skip the search.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os

import numpy as np

from . import _lib as L
from .solver import SweError, _BC, _PREC, _dp, _ghosted


class Ensemble:
    def __init__(self, sizes, lengths=None, g=9.80665, cfl=0.45, bc="reflecting",
                 precision="fp64", device=0):
        self._lib = L.lib()
        self.sizes = [(int(a), int(b)) for a, b in sizes]
        n = len(self.sizes)
        p = L.SweParams()
        self._lib.swe_params_default(ctypes.byref(p))
        p.g, p.cfl = g, cfl
        p.bc = _BC[bc] if isinstance(bc, str) else int(bc)
        p.precision = _PREC[precision] if isinstance(precision, str) else int(precision)
        p.device = device
        self.precision = precision
        nx = (ctypes.c_int * n)(*[s[0] for s in self.sizes])
        ny = (ctypes.c_int * n)(*[s[1] for s in self.sizes])
        lens = lengths or [(1.0, 1.0)] * n
        lx = (ctypes.c_double * n)(*[float(a) for a, _ in lens])
        ly = (ctypes.c_double * n)(*[float(b) for _, b in lens])
        self._ctx = ctypes.c_void_p()
        st = self._lib.swe_ens_create(ctypes.byref(p), n, nx, ny, lx, ly, ctypes.byref(self._ctx))
        if st != L.SWE_OK:
            self._ctx = ctypes.c_void_p()
            raise SweError(st, "swe_ens_create: " + self._lib.swe_status_string(st).decode())
        self.n = n

    def _check(self, st, what):
        if st != L.SWE_OK:
            msg = self._lib.swe_ens_last_error(self._ctx).decode() if self._ctx else ""
            raise SweError(st, f"{what}: {self._lib.swe_status_string(st).decode()}: {msg}")

    def close(self):
        if self._ctx:
            self._lib.swe_ens_destroy(self._ctx)
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

    def upload(self, q, h, hu, hv, B):
        Nx, Ny = self.sizes[q]
        arrs = [_ghosted(a, Nx, Ny, n) for a, n in ((h, "h"), (hu, "hu"), (hv, "hv"), (B, "B"))]
        self._check(self._lib.swe_ens_upload(self._ctx, q, *(_dp(a) for a in arrs)),
                    "swe_ens_upload")

    def download(self, q):
        Nx, Ny = self.sizes[q]
        out = tuple(np.empty((Nx + 4, Ny + 4)) for _ in range(3))
        self._check(self._lib.swe_ens_download(self._ctx, q, *(_dp(a) for a in out)),
                    "swe_ens_download")
        return out

    def step(self, n_steps=1, dt=None):
        self._check(self._lib.swe_ens_step(self._ctx, int(n_steps), float(dt or 0.0)),
                    "swe_ens_step")

    def times(self):
        t = np.zeros(self.n)
        self._check(self._lib.swe_ens_times(self._ctx, _dp(t)), "swe_ens_times")
        return t

    def last_dt(self):
        t = np.zeros(self.n)
        self._check(self._lib.swe_ens_last_dt(self._ctx, _dp(t)), "swe_ens_last_dt")
        return t

    def last_step_ms(self):
        v = ctypes.c_double()
        self._check(self._lib.swe_ens_last_step_ms(self._ctx, ctypes.byref(v)), "swe_ens_last_step_ms")
        return v.value

    def kernel_launches(self):
        return int(self._lib.swe_ens_kernel_launches(self._ctx))

    def schedule(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self._lib.swe_ens_get_schedule(self._ctx, ctypes.byref(a), ctypes.byref(b),
                                                   ctypes.byref(c)), "swe_ens_get_schedule")
        names = {v: k for k, v in L.SHAPES.items()}
        return {"shape": names[a.value], "grid": b.value, "tiles": c.value}

    def set_schedule(self, shape, grid):
        sid = L.SHAPES[shape] if isinstance(shape, str) else int(shape)
        self._check(self._lib.swe_ens_set_schedule(self._ctx, sid, int(grid)),
                    "swe_ens_set_schedule")

    def signature(self):
        h = hashlib.sha256(json.dumps([self.precision, sorted(self.sizes)]).encode()).hexdigest()
        return h[:16]

    def tune(self, steps=2, cache=None):
        """Runs the autotuner (or reuses a cached result for this signature)."""
        key = self.signature()
        if cache and os.path.exists(cache):
            try:
                entry = json.load(open(cache)).get(key)
            except (OSError, ValueError):
                entry = None
            if entry:
                self.set_schedule(entry["shape"], entry["grid"])
                return dict(entry, cached=True)
        best = ctypes.c_double()
        self._check(self._lib.swe_ens_tune(self._ctx, int(steps), ctypes.byref(best)), "swe_ens_tune")
        res = dict(self.schedule(), ms_per_step=best.value)
        if cache:
            data = {}
            if os.path.exists(cache):
                try:
                    data = json.load(open(cache))
                except (OSError, ValueError):
                    data = {}
            data[key] = res
            with open(cache, "w") as f:
                json.dump(data, f, indent=1)
        return dict(res, cached=False)
