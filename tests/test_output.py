"""NetCDF output written by the library's host path, checked against the reference
writers' data model (include/io/netCDF_writer.cpp:29-149,
include/io/sanity_checks_netcdf_writer.cpp:25-71) with two independent readers:
scipy.io.netcdf_file (CDF-2) and the grammar-level reader in tests/ncclassic.py
(CDF-2 and CDF-5).  The states are oracle runs; no GPU is used."""
from __future__ import annotations

import os

import numpy as np
import pytest

from ncclassic import ClassicFile

scipy_io = pytest.importorskip("scipy.io")

Nx, Ny, Lx, Ly = 19, 26, 2.0, 1.3
META = dict(dt=1.25e-3, backend="GB300", riemann_solver="HLL", reconstruction="MUSCL",
            time_integrator="SSPRK3", boundary_condition="Reflecting Walls",
            bathymetry="GaussianHill")


def oracle_records(port, problems, nrec=3, steps=4):
    """(B, [(t, h, hu, hv)]) of an oracle run with a snapshot every `steps` steps."""
    h, hu, hv, B = (np.array(a, dtype=np.float64) for a in problems.random_state(Nx, Ny, seed=11))
    p = port.grid(Nx, Ny, Lx, Ly)
    port.fill_ghosts(p, h, hu, hv)
    out, t = [(0.0, h, hu, hv)], 0.0
    for _ in range(nrec - 1):
        h, hu, hv, dts, dt_t, st = port.run(p, h, hu, hv, B, steps, META["dt"])
        assert st == 0
        t += dt_t
        out.append((t, h, hu, hv))
    return B, out


def write_file(sw, path, B, recs, fmt=0, units=("m", "m", "m", "s"), meta=META):
    w = sw.output.NetCDFWriter(path, (Nx, Ny, Lx, Ly), *units, save_every=4, format=fmt)
    w.write_bathymetry(B)
    for k, (t, h, hu, hv) in enumerate(recs):
        w.write_snapshot((h, hu, hv), t, **(meta if k == 0 else {}))
    assert w.records == len(recs)
    w.close()


def interior(a):
    return np.asarray(a)[2:-2, 2:-2]


def check_contents(get, dims, gatts, vatts, B, recs):
    """get(name) -> array as stored; dims / attribute dicts from one reader."""
    assert dims == {"time": len(recs), "x": Nx, "y": Ny}
    x, y = get("x"), get("y")
    dx, dy = Lx / Nx, Ly / Ny  # grid.hpp:19-23
    assert np.array_equal(x, np.array([(i + 0.5) * dx for i in range(Nx)]))
    assert np.array_equal(y, np.array([(j + 0.5) * dy for j in range(Ny)]))
    assert np.array_equal(get("B").view(np.uint64), interior(B).astype(">f8").view(np.uint64))
    assert np.array_equal(get("time"), np.array([r[0] for r in recs]))
    for f, name in enumerate(("h", "hu", "hv")):
        got = get(name)
        assert got.shape == (len(recs), Nx, Ny)
        for k, r in enumerate(recs):
            assert np.array_equal(got[k].astype(np.float64).view(np.uint64),
                                  interior(r[1 + f]).view(np.uint64)), (name, k)
    assert gatts["save_every"] == 4
    assert gatts["dt"] == META["dt"]
    for key in ("backend", "riemann_solver", "reconstruction", "time_integrator",
                "boundary_condition", "bathymetry"):
        assert gatts[key] == META[key]
    assert vatts["x"]["units"] == "m" and vatts["y"]["units"] == "m"
    assert vatts["h"]["units"] == "m" and vatts["B"]["units"] == "m"
    assert vatts["time"]["units"] == "s"
    assert "units" not in vatts["hu"] and "units" not in vatts["hv"]


def _text(v):
    return v.decode() if isinstance(v, bytes) else v


def test_snapshot_file_scipy(sw, port, problems, tmp_path):
    B, recs = oracle_records(port, problems)
    path = str(tmp_path / "out" / "snap.nc")  # parent directory is created
    write_file(sw, path, B, recs)
    with scipy_io.netcdf_file(path, "r", mmap=False) as f:
        assert f.version_byte == 2
        dims = {k: (len(recs) if v is None else v) for k, v in f.dimensions.items()}
        assert list(f.variables) == ["time", "x", "y", "h", "hu", "hv", "B"]
        assert f.variables["h"].dimensions == ("time", "x", "y")
        assert f.variables["B"].dimensions == ("x", "y")
        gatts = {k: _text(v) for k, v in f._attributes.items()}
        vatts = {n: {k: _text(a) for k, a in v._attributes.items()} for n, v in f.variables.items()}
        data = {n: np.array(v.data) for n, v in f.variables.items()}
    check_contents(lambda n: data[n], dims, gatts, vatts, B, recs)


@pytest.mark.parametrize("fmt", [2, 5])
def test_snapshot_file_grammar_reader(sw, port, problems, tmp_path, fmt):
    B, recs = oracle_records(port, problems)
    path = str(tmp_path / f"snap{fmt}.nc")
    write_file(sw, path, B, recs, fmt=fmt)
    f = ClassicFile(path)
    assert f.version == fmt and f.numrecs == len(recs)
    dims = {n: (f.numrecs if l == 0 else l) for n, l in f.dims}
    assert [n for n, _ in f.dims] == ["time", "x", "y"]
    gatts = {k: (v if isinstance(v, str) else v.item()) for k, v in f.gatts.items()}
    assert list(gatts) == ["save_every", "dt", "backend", "riemann_solver", "reconstruction",
                           "time_integrator", "boundary_condition", "bathymetry"]
    assert f.gatts["save_every"].dtype == np.dtype(">i4")
    vatts = {n: v["atts"] for n, v in f.vars.items()}
    assert all(v["type"] == 6 for v in f.vars.values())  # NC_DOUBLE
    check_contents(f.read, dims, gatts, vatts, B, recs)
    # the data section starts after the header and every begin is 4-byte aligned
    assert all(v["begin"] >= f.header_end and v["begin"] % 4 == 0 for v in f.vars.values())


def test_metadata_rules(sw, port, problems, tmp_path):
    """netCDF_writer.cpp:107-133: applied once, by the first call carrying dt or one of
    the strings after backend; backend alone does not trigger it; empty units give no
    attribute (:43-54)."""
    B, recs = oracle_records(port, problems, nrec=3)
    path = str(tmp_path / "meta.nc")
    w = sw.output.NetCDFWriter(path, (Nx, Ny, Lx, Ly), "", "", "", "", save_every=1)
    w.write_snapshot(recs[0][1:], 0.0, backend="only-backend")
    w.write_snapshot(recs[1][1:], recs[1][0], dt=0.5, backend="GB300")
    w.write_snapshot(recs[2][1:], recs[2][0], dt=0.25, riemann_solver="ignored")
    w.close()
    f = ClassicFile(path)
    assert set(f.gatts) == {"save_every", "dt", "backend"}
    assert f.gatts["dt"].item() == 0.5 and f.gatts["backend"] == "GB300"
    assert all(not v["atts"] for v in f.vars.values())
    # B never written: it reads as netCDF's default double fill value
    assert np.all(f.read("B") == 9.9692099683868690e36)


def test_sanity_records(sw, tmp_path):
    """SanityCheckNetCDFWriter: CDF-5 with a uint64 step; values and attributes."""
    path = str(tmp_path / "sanity" / "s.nc")
    w = sw.output.SanityCheckNetCDFWriter(path, "s", "m", 10, 2.5e-4, "GB300", "HLL", "MUSCL",
                                          "SSPRK3", "Reflecting Walls", "")
    rows = [(0, 0.0, 0.0, 0.5), (10, 2.5e-3, 1.25e-16, 0.4375), (2**40 + 3, 7.0, 3e-15, -0.0)]
    for r in rows:
        w.write(*r)
    w.close()
    f = ClassicFile(path)
    assert f.version == 5 and f.numrecs == 3
    assert [n for n, _ in f.dims] == ["record"] and f.dims[0][1] == 0
    assert list(f.vars) == ["step", "time", "mass_rel_err", "h_min"]
    assert f.vars["step"]["type"] == 11  # NC_UINT64
    assert f.read("step").tolist() == [r[0] for r in rows]
    for k, name in enumerate(("time", "mass_rel_err", "h_min"), start=1):
        got = f.read(name).astype(np.float64)
        assert np.array_equal(got.view(np.uint64), np.array([r[k] for r in rows]).view(np.uint64))
    v = f.vars
    assert v["step"]["atts"] == {"long_name": "time_step_index"}
    assert v["time"]["atts"] == {"long_name": "physical_time", "units": "s"}
    assert v["mass_rel_err"]["atts"] == {"long_name": "relative_mass_error", "units": "1"}
    assert v["h_min"]["atts"] == {"long_name": "minimum_water_height", "units": "m"}
    g = f.gatts
    assert list(g) == ["save_every", "dt", "backend", "riemann_solver", "reconstruction",
                       "time_integrator", "boundary_condition", "bathymetry",
                       "mass_conservation_enabled", "positivity_enabled"]
    assert g["save_every"].item() == 10 and g["dt"].item() == 2.5e-4
    assert g["bathymetry"] == "" and g["boundary_condition"] == "Reflecting Walls"
    assert g["mass_conservation_enabled"].item() == 1 and g["positivity_enabled"].item() == 1


def test_open_errors(sw, tmp_path):
    L = sw._lib
    blocker = tmp_path / "file"
    blocker.write_text("x")
    with pytest.raises(sw.SweError) as e:  # a parent that is a regular file
        sw.output.NetCDFWriter(str(blocker / "a.nc"), (4, 4, 1.0, 1.0))
    assert e.value.status == L.SWE_ERR_IO
    with pytest.raises(sw.SweError) as e:  # 5.2 GB per field cannot be described in CDF-2
        sw.output.NetCDFWriter(str(tmp_path / "big.nc"), (25600, 25600, 1.0, 1.0), format=2)
    assert e.value.status == L.SWE_ERR_BAD_ARG
    assert not os.path.exists(tmp_path / "big.nc")
    with pytest.raises(sw.SweError) as e:
        sw.output.NetCDFWriter(str(tmp_path / "bad.nc"), (4, 4, 1.0, 1.0), format=3)
    assert e.value.status == L.SWE_ERR_BAD_ARG

