"""Minimal reader of netCDF classic files (CDF-1, CDF-2, CDF-5) for the output tests.

Written from the published classic-format grammar, independently of the library's
writer: it parses the header into dimensions, global attributes and variables, and
reads a variable's data with numpy (big-endian).  scipy.io.netcdf_file covers CDF-1/2
as a second, third-party reader; this one also reads CDF-5, which scipy does not.
"""
from __future__ import annotations

import numpy as np

_TYPES = {1: ">i1", 2: "S1", 3: ">i2", 4: ">i4", 5: ">f4", 6: ">f8", 7: ">u1", 8: ">u2",
          9: ">u4", 10: ">i8", 11: ">u8"}


class ClassicFile:
    def __init__(self, path: str):
        self.path = path
        with open(path, "rb") as f:
            self.raw = f.read()
        self.pos = 0
        magic = self.raw[:3]
        if magic != b"CDF":
            raise ValueError("not a classic netCDF file")
        self.version = self.raw[3]
        self.pos = 4
        self.nn = 8 if self.version == 5 else 4
        self.off = 4 if self.version == 1 else 8
        self.numrecs = self._nn()
        self.dims = []  # (name, length)
        tag = self._u32()
        n = self._nn()
        if tag == 0x0A:
            for _ in range(n):
                self.dims.append((self._name(), self._nn()))
        elif (tag, n) != (0, 0):
            raise ValueError("bad dim_list")
        self.gatts = self._atts()
        self.vars = {}
        tag = self._u32()
        n = self._nn()
        if tag == 0x0B:
            for _ in range(n):
                name = self._name()
                nd = self._nn()
                dimids = [self._nn() for _ in range(nd)]
                atts = self._atts()
                typ = self._u32()
                vsize = self._nn()
                begin = self._u(self.off)
                self.vars[name] = dict(dimids=dimids, atts=atts, type=typ, vsize=vsize,
                                       begin=begin)
        elif (tag, n) != (0, 0):
            raise ValueError("bad var_list")
        self.header_end = self.pos
        self.recsize = sum(v["vsize"] for v in self.vars.values() if self._is_rec(v))

    def _u(self, n):
        v = int.from_bytes(self.raw[self.pos:self.pos + n], "big")
        self.pos += n
        return v

    def _u32(self):
        return self._u(4)

    def _nn(self):
        return self._u(self.nn)

    def _pad(self):
        self.pos += (-self.pos) % 4

    def _name(self):
        n = self._nn()
        s = self.raw[self.pos:self.pos + n].decode()
        self.pos += n
        self._pad()
        return s

    def _atts(self):
        tag = self._u32()
        n = self._nn()
        out = {}
        if tag == 0x0C:
            for _ in range(n):
                name = self._name()
                typ = self._u32()
                ne = self._nn()
                dt = np.dtype(_TYPES[typ])
                b = self.raw[self.pos:self.pos + ne * dt.itemsize]
                self.pos += ne * dt.itemsize
                self._pad()
                out[name] = b.decode() if typ == 2 else np.frombuffer(b, dt).copy()
        elif (tag, n) != (0, 0):
            raise ValueError("bad att_list")
        return out

    def _is_rec(self, v):
        return bool(v["dimids"]) and self.dims[v["dimids"][0]][1] == 0

    def shape(self, name):
        v = self.vars[name]
        return tuple(self.numrecs if self.dims[d][1] == 0 else self.dims[d][1]
                     for d in v["dimids"])

    def read(self, name) -> np.ndarray:
        v = self.vars[name]
        dt = np.dtype(_TYPES[v["type"]])
        shp = self.shape(name)
        if not self._is_rec(v):
            n = int(np.prod(shp)) if shp else 1
            return np.frombuffer(self.raw, dt, n, v["begin"]).reshape(shp).copy()
        per = int(np.prod(shp[1:])) if len(shp) > 1 else 1
        recs = [np.frombuffer(self.raw, dt, per, v["begin"] + r * self.recsize)
                for r in range(self.numrecs)]
        return np.stack(recs).reshape(shp) if recs else np.zeros(shp, dt)
