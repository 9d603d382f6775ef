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
import sys
import time

import numpy as np

from .inputs import InputError, read_geom, read_inputs
from .records import DumpWriter
from .solver import QMSSolver, default_desc
from .trajectory import VelocitySchedule, scaled_field


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
    try:
        solver.set_geometry_f64(geom, inp.props_table())
        writer = DumpWriter(inp, workdir)
        log("Setup completed in {:6.2f} seconds.".format(time.time() - t0))
        log("Intializing steady state...")
        t1 = time.time()
        sched = VelocitySchedule(inp.traj, inp.dt)
        B, G = scaled_field(inp.B, inp.G, inp.excitation, 0.0)
        stats.append(solver.steady(sched.steady(), B, G))
        _dump(solver, writer, inp, 0)
        log("Initialization of steady state completed in {:6.2f} seconds.".format(time.time() - t1))
        log("Starting main time marching algorithm...")
        t2 = time.time()
        for counter in range(1, inp.nt + 1):
            v = sched.step(counter)
            B, G = scaled_field(inp.B, inp.G, inp.excitation, counter * inp.dt)
            stats.append(solver.step(v, B, G))
            if counter % 10 == 0:
                log(f"{counter} of {inp.nt} time steps")
            _dump(solver, writer, inp, counter)
        writer.close()
        log("Main time marching completed in {:6.2f} seconds.".format(time.time() - t2))
    finally:
        solver.close()
    return stats


def _dump(solver, writer, inp, counter):
    if writer.wants_slice(counter):
        writer.write_slice(solver.slices(inp.slice_axis, inp.slice_index))
    if inp.save_all_fields:
        writer.write_cube(solver.fields())


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
