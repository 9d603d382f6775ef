"""Golden fixture for the 32^3 copper-block workload (steady + 20 steps at 1 kHz).

The CPU oracle (C assembly + row-equilibrated SuperLU with refinement) takes
minutes at this size, so its results are stored here once:
tests/golden/plain_block_32.npz holds, for the steady state and every step,
the three H components on the z-mid slice (the record the drop-in writes to
Hx.bin / Hy.bin / Hz.bin) and the norms of A and of the full H cubes; and, for
the steps in FULL_STEPS, the whole A block, the edge current sigma grad V and
the three H cubes, so that those steps are compared vector by vector.

Usage:  python tests/golden/make_config1.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import qms_oracle as o  # noqa: E402
from alpineqms_gb300 import workloads  # noqa: E402


FULL_STEPS = (1, 20)


def main():
    inp, geom = workloads.plain_block_32()
    p = dict(xs=inp.xs, ys=inp.ys, zs=inp.zs, dx=inp.dx, dy=inp.dy, dz=inp.dz, dt=inp.dt, Nt=inp.nt, B=inp.B,
             G=inp.G, traj=[(t.v0, t.accel, t.n_accel) for t in inp.traj], props=inp.props_table(),
             excitation=inp.excitation)
    states = o.simulate(p, geom, keep_states=True)
    oV = o.block_offsets(inp.xs, inp.ys, inp.zs)[3]
    sl = inp.slice_index - 1
    c = o.materials(inp.xs, inp.ys, inp.zs, geom, inp.props_table())
    slices, anorm, hnorm = [], [], []
    full = {}
    for counter, x, H in states:
        if counter in FULL_STEPS:
            full["a_%d" % counter] = x[:oV]
            full["j_%d" % counter] = o.edge_current_from_v(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, x)
            full["h_%d" % counter] = np.concatenate(H)
        cubes = [h.reshape((inp.xs, inp.ys, inp.zs), order="F") for h in H]
        slices.append(np.stack([c[:, :, sl] for c in cubes]))
        anorm.append(np.linalg.norm(x[:oV]))
        hnorm.append(np.sqrt(sum(np.dot(h, h) for h in H)))
    np.savez_compressed(os.path.join(HERE, "plain_block_32.npz"), slices=np.array(slices),
                        anorm=np.array(anorm), hnorm=np.array(hnorm), slice_index=inp.slice_index,
                        full_steps=np.array(FULL_STEPS), **full)
    print("records", len(slices))


if __name__ == "__main__":
    main()
