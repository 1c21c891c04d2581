"""The C ABI library loads on any machine and exports every symbol include/*.h declares;
argument checking works without a GPU (no compute call is made here)."""
from __future__ import annotations

import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(hdr).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]*?\b(swe_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol(sw):
    L = sw.lib()
    names = declared_symbols()
    assert len(names) >= 12
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) <= set(sw._lib.EXPORTS) | set(names)


def test_params_default(sw):
    L = sw.lib()
    p = sw._lib.SweParams()
    L.swe_params_default(ctypes.byref(p))
    assert (p.nG, p.Lx, p.Ly, p.g, p.cfl, p.bc, p.precision) == (2, 1.0, 1.0, 9.80665, 0.45, 0, 0)
    assert (p.scheme, p.reconstruction, p.riemann, p.bathymetry) == (0, 1, 0, 1)


def test_struct_layouts_match_the_binding(sw):
    L = sw.lib()
    assert L.swe_params_size() == ctypes.sizeof(sw._lib.SweParams)
    assert L.swe_snapshot_params_size() == ctypes.sizeof(sw._lib.SnapshotParams)


@pytest.mark.parametrize("field,value", [("nG", 1), ("Nx", 1), ("Ny", 0), ("Lx", 0.0),
                                         ("cfl", -1.0), ("bc", 7)])
def test_create_rejects_bad_params(sw, field, value):
    L = sw.lib()
    p = sw._lib.SweParams()
    L.swe_params_default(ctypes.byref(p))
    p.Nx, p.Ny = 16, 16
    setattr(p, field, value)
    ctx = ctypes.c_void_p()
    assert L.swe_create(ctypes.byref(p), ctypes.byref(ctx)) == sw._lib.SWE_ERR_BAD_ARG
    assert not ctx.value


def test_null_context_calls_are_safe(sw):
    L = sw.lib()
    assert L.swe_step(None, 1, 0.0, None) == sw._lib.SWE_ERR_BAD_ARG
    assert L.swe_step_host(None, None, None, None, None, None, None, None, 1, 0.0,
                           None) == sw._lib.SWE_ERR_BAD_ARG
    assert L.swe_status_string(3) == b"non-finite state detected"
    L.swe_destroy(None)
