"""Field dumps in the reference's format (3D/QMS_3D.f90:407-417, F:1378-1404, F:2274-2300).

The reference opens ``Hx.bin``, ``Hy.bin``, ``Hz.bin`` (and, when
``save_all_fields`` is ``yes``, ``Hx_all.bin`` ...) as Fortran unformatted
sequential files.  Each ``write`` is one record: a 4-byte little-endian length
marker, the float64 payload in Fortran (column-major) order, the same marker
again.  plot.py:141-160 and paraview_time.py:29-47 read these records with
``scipy.io.FortranFile.read_reals(float64)``.

Cadence (F:1379, F:2275, F:2296): the slice record is written when
``mod(counter, tt) == 0`` with ``counter = 0`` for the steady state, so the
steady slice is always written and ``1 + Nt // tt`` slice records result; the
full cube is written for the steady state and every step (``tt`` ignored).
"""
from __future__ import annotations

import os
import struct

import numpy as np


def record_bytes(arr: np.ndarray) -> bytes:
    data = np.asarray(arr, dtype="<f8").tobytes(order="F")
    m = struct.pack("<i", len(data))
    return m + data + m


def read_records(path: str, shape=None):
    """Reader used by tests (same contract as plot.py's FortranFile loop)."""
    out = []
    with open(path, "rb") as f:
        buf = f.read()
    pos = 0
    while pos + 4 <= len(buf):
        (n,) = struct.unpack_from("<i", buf, pos)
        rec = np.frombuffer(buf, dtype="<f8", count=n // 8, offset=pos + 4).copy()
        (n2,) = struct.unpack_from("<i", buf, pos + 4 + n)
        if n2 != n:
            raise ValueError("corrupt record markers")
        pos += 8 + n
        out.append(rec if shape is None else rec.reshape(shape, order="F"))
    return out


class DumpWriter:
    """Writes the H dumps with the reference's file names and cadence."""

    def __init__(self, inp, directory: str = "."):
        self.inp = inp
        self.slice_files = [open(os.path.join(directory, f"H{c}.bin"), "wb") for c in "xyz"]
        self.cube_files = ([open(os.path.join(directory, f"H{c}_all.bin"), "wb") for c in "xyz"]
                           if inp.save_all_fields else [])

    def wants_slice(self, counter: int) -> bool:
        return counter % self.inp.tt == 0

    def write_slice(self, slices):
        """slices: three 2-D arrays in (first, second) slice order (F:1380-1394)."""
        for f, s in zip(self.slice_files, slices):
            f.write(record_bytes(s))

    def write_cube(self, cubes):
        """cubes: three (xs, ys, zs) arrays (F:1400-1404)."""
        for f, c in zip(self.cube_files, cubes):
            f.write(record_bytes(c))

    def close(self):
        for f in self.slice_files + self.cube_files:
            f.close()


def slice_of(cube: np.ndarray, axis: str, index: int) -> np.ndarray:
    """Hx(location,1:ys,1:zs) etc.; `cube` is (xs, ys, zs), index is 1-based (F:1380-1394)."""
    if axis == "x":
        return cube[index - 1, :, :]
    if axis == "y":
        return cube[:, index - 1, :]
    return cube[:, :, index - 1]
