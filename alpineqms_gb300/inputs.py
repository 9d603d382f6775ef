"""``inputs.txt`` / ``geom.bin`` reader: the boundary contract of QMS_3D.

The reference solver is driven by 3D/master.py:16-84, which writes a
positional, list-directed ``inputs.txt`` and a raw float64 ``geom.bin`` and
then runs ``./QMS_3D inputs.txt``.  This module reads both exactly as the
Fortran program does (3D/QMS_3D.f90:120-165, F:229-254):

* one ``read(1,*)`` per item, values separated by commas and/or blanks, a
  record continuing onto the next line if it holds too few values, the rest
  of the last line read being skipped;
* ``num_materials`` triples of lines (ID, mu_r xyz, sigma xyz);
* the geometry file name, after which the reference closes the file
  (F:163-165), so trailing lines are ignored by the reference.

Extension (ignored by the reference, so files stay reference-compatible): an
optional trailing line ``excitation,<cos|sin>,<f_Hz>[,<phase_rad>]`` scales
the whole background field B_in + G.r by s(t) = cos(2 pi f t + phase) (or sin)
at t = n*dt for step n (t = 0 for the steady state).

Extension (trajectory types the reference rejects with STOP, F:135-151; a file
using them is therefore not one the reference runs): per axis, after the type
line,

* type 2, harmonic motion: one record ``amplitude, f_Hz, phase_rad``, the frame
  velocity being v(n) = amplitude * sin(2 pi f n dt + phase);
* type 3, a velocity table: a record ``n_points`` and then a record of that
  many velocities (which may continue over several lines), v(n) = table[min(n,
  n_points - 1)] for the steady state (n = 0) and each step n.

Errors the reference reports with STOP (any other trajectory type,
F:135-151) raise ``InputError`` with the same message.  Inputs on which the
reference has undefined behaviour (slice axis not x/y/z, slice index out of
range, tt <= 0, geometry IDs above the largest table ID or negative, no
materials) are rejected up front with an ``InputError``.
"""
from __future__ import annotations

import dataclasses
import os
import re
from typing import List, Optional, Tuple

import numpy as np

MU0 = 1.25663706e-6  # 3D/QMS_3D.f90:22


class InputError(ValueError):
    pass


@dataclasses.dataclass
class Material:
    mat_id: float                       # material_properties(i,1,1) (read as a real, used via int())
    mu_r: Tuple[float, float, float]    # material_properties(i,2,1..3)
    sigma: Tuple[float, float, float]   # material_properties(i,3,1..3)


@dataclasses.dataclass
class Trajectory:
    """One axis of the frame motion.  Type 1 (the reference's, F:136-137) uses v0, accel and
    n_accel; type 2 (harmonic) amp, freq and phase; type 3 (velocity table) table."""
    kind: int
    v0: float = 0.0
    accel: float = 0.0
    n_accel: int = 0
    amp: float = 0.0
    freq: float = 0.0
    phase: float = 0.0
    table: Tuple[float, ...] = ()


@dataclasses.dataclass
class QMSInputs:
    xs: int
    ys: int
    zs: int
    dx: float
    dy: float
    dz: float
    dt: float
    nt: int
    tt: int
    slice_axis: str
    slice_index: int
    save_all: str
    B: Tuple[float, float, float]
    G: Tuple[Tuple[float, float, float], ...]
    traj: Tuple[Trajectory, Trajectory, Trajectory]
    materials: List[Material]
    geom_name: str
    excitation: Optional[Tuple[str, float, float]] = None

    @property
    def save_all_fields(self) -> bool:
        return self.save_all.strip() == "yes"    # F:413 TRIM(save_all_fields)=='yes'

    def props_table(self) -> np.ndarray:
        """(nmat, 7) float64: id, mu_r xyz, sigma xyz."""
        return np.array([[m.mat_id, *m.mu_r, *m.sigma] for m in self.materials], dtype=np.float64).reshape(-1, 7)

    @property
    def G_flat(self) -> np.ndarray:
        return np.array(self.G, dtype=np.float64).reshape(9)

    @property
    def n_dims(self) -> int:
        Nx, Ny, Nz = self.xs + 1, self.ys + 1, self.zs + 1
        return 4 * Nx * Ny * Nz - Ny * Nz - Nx * Nz - Nx * Ny

    def slice_shape(self) -> Tuple[int, int]:
        return {"x": (self.ys, self.zs), "y": (self.xs, self.zs), "z": (self.xs, self.ys)}[self.slice_axis]


class _ListReader:
    """Fortran list-directed record reader over the lines of a text file."""

    def __init__(self, text: str):
        self.lines = text.splitlines()
        self.pos = 0

    def read(self, count: int, what: str) -> List[str]:
        vals: List[str] = []
        while len(vals) < count:
            if self.pos >= len(self.lines):
                raise InputError(f"inputs file ended while reading {what}")
            line = self.lines[self.pos]
            self.pos += 1
            for tok in re.split(r"[,\s]+", line.strip()):
                if tok == "":
                    continue
                if tok.startswith("/"):
                    raise InputError(f"'/' terminator while reading {what} is not supported")
                vals.append(tok.strip("'\""))
                if len(vals) == count:
                    break
        return vals

    def rest(self) -> List[str]:
        return self.lines[self.pos:]


def _f(tok: str, what: str) -> float:
    try:
        return float(tok.replace("d", "e").replace("D", "e"))
    except ValueError:
        raise InputError(f"bad real value {tok!r} for {what}") from None


def _i(tok: str, what: str) -> int:
    if not re.fullmatch(r"[+-]?\d+", tok):
        raise InputError(f"bad integer value {tok!r} for {what}")
    return int(tok)


def parse_inputs_text(text: str) -> QMSInputs:
    r = _ListReader(text)
    xs, ys, zs = (_i(t, "grid size") for t in r.read(3, "grid size"))        # F:123
    dx, dy, dz = (_f(t, "grid step") for t in r.read(3, "grid step"))        # F:124
    dt = _f(r.read(1, "del_t")[0], "del_t")                                   # F:125
    nt = _i(r.read(1, "time_steps")[0], "time_steps")                         # F:126
    tt = _i(r.read(1, "tt")[0], "tt")                                         # F:127
    ax, loc = r.read(2, "output slice")                                       # F:128
    ax = ax[:3]                                                               # character(3)
    loc = _i(loc, "slice location")
    save_all = r.read(1, "save_all_fields")[0][:3]                            # F:129
    B = tuple(_f(t, "B_in") for t in r.read(3, "B_in"))                      # F:130
    G = tuple(tuple(_f(t, "gradient") for t in r.read(3, "gradient")) for _ in range(3))  # F:131-133
    trajs = []
    for axis in "XYZ":                                                        # F:134-151
        kind = _i(r.read(1, "trajectory type")[0], "trajectory type")
        if kind == 1:
            v0, a, n = r.read(3, "trajectory")
            trajs.append(Trajectory(kind, _f(v0, "initial velocity"), _f(a, "acceleration"),
                                    _i(n, "acceleration steps")))
        elif kind == 2:
            amp, f, ph = r.read(3, "harmonic trajectory")
            trajs.append(Trajectory(kind, amp=_f(amp, "velocity amplitude"), freq=_f(f, "motion frequency"),
                                    phase=_f(ph, "motion phase")))
        elif kind == 3:
            npts = _i(r.read(1, "velocity table length")[0], "velocity table length")
            if npts < 1:
                raise InputError(f"velocity table in {axis} direction needs at least one value")
            table = tuple(_f(t, "velocity table") for t in r.read(npts, "velocity table"))
            trajs.append(Trajectory(kind, table=table))
        else:
            raise InputError(f"ERROR: TYPE OF TRAJECTORY IN {axis} DIRECTION IS NOT SUPPORTED")
    nmat = _i(r.read(1, "num_materials")[0], "num_materials")                 # F:153
    mats = []
    for _ in range(max(nmat, 0)):                                             # F:157-161
        mid = _f(r.read(1, "material ID")[0], "material ID")
        mu = tuple(_f(t, "mu_r") for t in r.read(3, "mu_r"))
        sg = tuple(_f(t, "sigma") for t in r.read(3, "sigma"))
        mats.append(Material(mid, mu, sg))
    geom_name = r.read(1, "geometry file name")[0]                           # F:163
    exc = None
    for line in r.rest():                                                     # ignored by the reference
        toks = [t for t in re.split(r"[,\s]+", line.strip()) if t]
        if toks and toks[0].lower() == "excitation":
            if len(toks) < 3 or toks[1].lower() not in ("cos", "sin"):
                raise InputError("excitation line must be: excitation,<cos|sin>,<f_Hz>[,<phase_rad>]")
            exc = (toks[1].lower(), _f(toks[2], "excitation frequency"),
                   _f(toks[3], "excitation phase") if len(toks) > 3 else 0.0)
    inp = QMSInputs(xs, ys, zs, dx, dy, dz, dt, nt, tt, ax.strip(), loc, save_all, B, G, tuple(trajs),
                    mats, geom_name, exc)
    validate(inp)
    return inp


def validate(inp: QMSInputs) -> None:
    if min(inp.xs, inp.ys, inp.zs) < 4:
        raise InputError("grid must have at least 4 cells per axis (two-layer Dirichlet shell, F:361-396)")
    if inp.slice_axis not in ("x", "y", "z"):
        raise InputError(f"output slice axis must be x, y or z (got {inp.slice_axis!r})")
    lim = {"x": inp.xs, "y": inp.ys, "z": inp.zs}[inp.slice_axis]
    if not 1 <= inp.slice_index <= lim:
        raise InputError(f"slice index {inp.slice_index} outside 1..{lim}")
    if inp.tt <= 0:
        raise InputError("tt (save stride) must be positive")
    if inp.nt < 0:
        raise InputError("time_steps must be >= 0")
    if not inp.materials:
        raise InputError("at least one material is required (the reference reads the table maximum, F:234)")
    if len(inp.materials) > 255:
        raise InputError("at most 255 materials are supported (uint8 material slots)")
    for m in inp.materials:
        if int(m.mat_id) < 0:
            raise InputError("material IDs must be non-negative")
        if int(m.mat_id) > 1 << 24:
            raise InputError("material IDs above 2^24 are not supported")
    if inp.dt <= 0 or min(inp.dx, inp.dy, inp.dz) <= 0:
        raise InputError("dt, dx, dy, dz must be positive")


def read_inputs(path: str) -> QMSInputs:
    with open(path) as f:
        return parse_inputs_text(f.read())


def read_geom(path: str, inp: QMSInputs) -> np.ndarray:
    """geom.bin: xs*ys*zs float64 (native little-endian), Fortran order (F:229-232)."""
    n = inp.xs * inp.ys * inp.zs
    if not os.path.exists(path):
        raise InputError(f"geometry file {path!r} not found")
    data = np.fromfile(path, dtype="<f8", count=n)
    if data.size < n:
        raise InputError(f"geometry file {path!r} holds {data.size} values, need {n}")
    return data


def material_index(geom: np.ndarray, inp: QMSInputs) -> np.ndarray:
    """float64 IDs -> uint8 material slot (0 = vacuum, r = table row r), F:234-254.

    An ID absent from the table maps to vacuum like the reference's
    temp_mat_id lookup; an ID above the table maximum, or negative, is an
    out-of-bounds access in the reference and is rejected here.  When several
    table rows share an ID the last one wins (F:236-238)."""
    ids = np.trunc(np.asarray(geom, dtype=np.float64)).astype(np.int64)
    maxid = max(int(m.mat_id) for m in inp.materials)
    if ids.size and (ids.min() < 0 or ids.max() > maxid):
        raise InputError("geometry holds a material ID that is negative or above the largest table ID")
    lut = np.zeros(maxid + 1, dtype=np.uint8)
    for r, m in enumerate(inp.materials):
        lut[int(m.mat_id)] = r + 1
    return lut[ids]
