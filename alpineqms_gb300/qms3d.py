"""Drop-in replacement of the QMS_3D executable.

3D/master.py:84 runs ``./QMS_3D inputs.txt`` in its working directory; this
module implements the same program on the GPU:

    python -m alpineqms_gb300.qms3d inputs.txt      (or the ``QMS_3D`` launcher)

Program flow (3D/QMS_3D.f90): read inputs.txt and geom.bin (F:117-165,
F:229-232); build the material coefficients (F:193-279); steady-state solve
at the t = 0 velocity (F:430-1317); H at cell centres and the dumps
(F:1319-1404); then ``Nt`` backward-Euler steps (F:1424-2302), each writing
the slice every ``tt`` steps and the full cube every step when requested.
The stdout messages follow the reference's (F:118, F:425-427, F:1412-1414,
F:2270-2272, F:2321-2322).
"""
from __future__ import annotations

import os
import queue
import sys
import threading
import time

import numpy as np

from ._lib import QMS_FIELD_CUBES, QMS_FIELD_SLICE
from .inputs import InputError, read_geom, read_inputs
from .records import DumpWriter
from .solver import PinnedBuffer, QMSSolver, default_desc
from .trajectory import VelocitySchedule, scaled_field


class AsyncDumps:
    """The per-step dumps (F:1378-1404, F:2274-2300) with their device-to-host copies overlapped
    with the next step: H is formed on the solver's stream and copied into one of two pinned
    buffers per field kind on a copy stream; a writer thread waits for each copy and writes the
    Fortran records in order while the main thread already steps on.  At most one record per
    kind is in flight, so a slow disk holds the solve back by one step at most."""

    SLICE_SLOTS, CUBE_SLOTS = (0, 1), (2, 3)

    def __init__(self, solver, writer, inp):
        self.solver, self.writer, self.inp = solver, writer, inp
        self.n1, self.n2 = solver.slice_shape(inp.slice_axis)
        self.ncell = inp.xs * inp.ys * inp.zs
        self.bufs = {q: PinnedBuffer(3 * self.n1 * self.n2) for q in self.SLICE_SLOTS}
        if inp.save_all_fields:
            self.bufs.update({q: PinnedBuffer(3 * self.ncell) for q in self.CUBE_SLOTS})
        self.free = {q: threading.Semaphore(1) for q in self.bufs}
        self.turn = {"slice": 0, "cube": 0}
        self.q = queue.Queue()
        self.error = None
        self.thread = threading.Thread(target=self._work, daemon=True)
        self.thread.start()

    def _issue(self, kind, which, slots, axis, index):
        slot = slots[self.turn[kind] % len(slots)]
        self.turn[kind] += 1
        self.free[slot].acquire()           # the writer has written this buffer's last record
        if self.error is not None:
            self.free[slot].release()
            raise self.error
        self.solver.fields_async(which, axis, index, self.bufs[slot], slot)
        self.q.put((kind, slot))

    def dump(self, counter):
        if self.writer.wants_slice(counter):
            self._issue("slice", QMS_FIELD_SLICE, self.SLICE_SLOTS, self.inp.slice_axis, self.inp.slice_index)
        if self.inp.save_all_fields:
            self._issue("cube", QMS_FIELD_CUBES, self.CUBE_SLOTS, "x", 1)

    def _work(self):
        while True:
            item = self.q.get()
            if item is None:
                return
            kind, slot = item
            try:
                if self.error is None:
                    self.solver.fields_sync(slot)
                    a = self.bufs[slot].array
                    if kind == "slice":
                        m = self.n1 * self.n2
                        self.writer.write_slice([a[q * m:(q + 1) * m].reshape((self.n1, self.n2), order="F")
                                                 for q in range(3)])
                    else:
                        m = self.ncell
                        shape = (self.inp.xs, self.inp.ys, self.inp.zs)
                        self.writer.write_cube([a[q * m:(q + 1) * m].reshape(shape, order="F") for q in range(3)])
            except Exception as e:   # reported by close() / the next dump
                self.error = e
            finally:
                self.free[slot].release()

    def close(self):
        if self.thread is not None:
            self.q.put(None)
            self.thread.join()
            self.thread = None
            for b in self.bufs.values():
                b.close()
        if self.error is not None:
            e, self.error = self.error, None
            raise e


def run(inputs_path: str, workdir: str = None, precision: str = "mixed", device: int = 0, log=print, **solver_kw):
    workdir = workdir or os.path.dirname(os.path.abspath(inputs_path))
    t0 = time.time()
    log("Reading in the inputs file and setting up the simulation...")
    inp = read_inputs(inputs_path)
    geom = read_geom(os.path.join(workdir, inp.geom_name), inp)
    desc = default_desc(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, inp.dt, precision=precision, device=device,
                        **solver_kw)
    solver = QMSSolver(desc)
    stats = []
    dumps = None
    try:
        solver.set_geometry_f64(geom, inp.props_table())
        writer = DumpWriter(inp, workdir)
        dumps = AsyncDumps(solver, writer, inp)
        log("Setup completed in {:6.2f} seconds.".format(time.time() - t0))
        log("Intializing steady state...")
        t1 = time.time()
        sched = VelocitySchedule(inp.traj, inp.dt)
        B, G = scaled_field(inp.B, inp.G, inp.excitation, 0.0)
        stats.append(solver.steady(sched.steady(), B, G))
        dumps.dump(0)
        log("Initialization of steady state completed in {:6.2f} seconds.".format(time.time() - t1))
        log("Starting main time marching algorithm...")
        t2 = time.time()
        for counter in range(1, inp.nt + 1):
            v = sched.step(counter)
            B, G = scaled_field(inp.B, inp.G, inp.excitation, counter * inp.dt)
            stats.append(solver.step(v, B, G))
            if counter % 10 == 0:
                log(f"{counter} of {inp.nt} time steps")
            dumps.dump(counter)
        dumps.close()
        writer.close()
        log("Main time marching completed in {:6.2f} seconds.".format(time.time() - t2))
    finally:
        if dumps is not None and dumps.thread is not None:
            dumps.q.put(None)          # a failed run: stop the writer before the handle goes
            dumps.thread.join()
            dumps.thread = None
        solver.close()
    return stats


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if not argv:
        print("usage: QMS_3D inputs.txt", file=sys.stderr)
        return 2
    try:
        run(argv[0], workdir=os.getcwd())
    except InputError as e:
        print(str(e))
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
