"""Reader of the binary restart, forcing and output files (numpy only, no
library or GPU needed).

Container (little-endian): a 128-byte header, a directory of 48-byte field
entries from byte 128, and from byte 4096 the records; every record holds
each field as one [width][mp] block in caller tile order.  The library
writes these files (cablegpu_restart_write, cablegpu_forcing_file_write,
cablegpu_run_forcing_file); this module reads them for analysis, and the
tests use it to check the library's writer byte by byte.
"""
from __future__ import annotations

import os

import numpy as np

MAGIC = b"CABLEGPU"
VERSION = 1
DATA_OFFSET = 4096
KINDS = {1: "restart", 2: "forcing", 3: "output"}
F32, F64, I32, DF32 = 0, 1, 2, 3

HEADER = np.dtype([("magic", "S8"), ("version", "<u4"), ("kind", "<u4"), ("mp", "<u8"), ("nfields", "<u4"),
                   ("nrecords", "<u4"), ("ktau", "<i4"), ("doy0", "<i4"), ("dels", "<f4"), ("reserved0", "<u4"),
                   ("data_offset", "<u8"), ("record_bytes", "<u8"), ("reserved", "u1", (64,))])
ENTRY = np.dtype([("name", "S32"), ("dtype", "<u4"), ("width", "<u4"), ("offset", "<u8")])
assert HEADER.itemsize == 128 and ENTRY.itemsize == 48


class CgFile:
    """A parsed file: ``header`` (dict), ``fields`` (name -> (dtype, width,
    offset)) and ``read(name, record=0)``."""

    def __init__(self, path):
        self.path = path
        raw = np.fromfile(path, np.uint8, count=DATA_OFFSET)
        if raw.size < 128:
            raise ValueError("%s: too short for a CABLEGPU header" % path)
        h = raw[:128].view(HEADER)[0]
        if bytes(h["magic"]) != MAGIC:
            raise ValueError("%s: not a CABLEGPU file (bad magic)" % path)
        if int(h["version"]) != VERSION:
            raise ValueError("%s: unsupported version %d" % (path, int(h["version"])))
        self.header = {k: (h[k].item() if k != "magic" else bytes(h[k])) for k in HEADER.names if k != "reserved"}
        self.mp = int(h["mp"])
        n = int(h["nfields"])
        ents = raw[128:128 + 48 * n].view(ENTRY)
        self.fields = {bytes(e["name"]).rstrip(b"\0").decode(): (int(e["dtype"]), int(e["width"]), int(e["offset"]))
                       for e in ents}
        need = DATA_OFFSET + int(h["record_bytes"]) * int(h["nrecords"])
        if os.path.getsize(path) < need:
            raise ValueError("%s: file shorter than its records (truncated)" % path)

    @property
    def kind(self) -> str:
        return KINDS.get(self.header["kind"], "unknown")

    def read(self, name, record: int = 0) -> np.ndarray:
        """Field ``name`` of ``record``: [width][mp] (f32, f64 or i32);
        double-FP32 fields are returned as their FP64 values and their word
        pairs are available through ``read_pairs``."""
        dt, w, off = self.fields[name]
        if dt == DF32:
            hi, lo = self.read_pairs(name, record)
            return hi.astype(np.float64) + lo.astype(np.float64)
        npdt = {F32: "<f4", F64: "<f8", I32: "<i4"}[dt]
        return self._block(record, off, npdt, w)

    def read_pairs(self, name, record: int = 0):
        dt, w, off = self.fields[name]
        assert dt == DF32
        words = self._block(record, off, "<f4", 2 * w)
        return words[:w], words[w:]

    def _block(self, record, off, npdt, rows):
        rb = int(self.header["record_bytes"])
        if not 0 <= record < int(self.header["nrecords"]):
            raise IndexError("record %d of %d" % (record, self.header["nrecords"]))
        start = DATA_OFFSET + rb * record + off
        a = np.fromfile(self.path, np.dtype(npdt), count=rows * self.mp, offset=start)
        if a.size != rows * self.mp:
            raise ValueError("%s: truncated record %d" % (self.path, record))
        return a.reshape(rows, self.mp)


def read(path) -> CgFile:
    return CgFile(path)
