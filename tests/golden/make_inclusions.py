"""Golden fixture for the random-inclusion workload at 32^3 (24 ellipsoids, mu_r
log-uniform in [1, 1e3], sigma log-uniform in [1e5, 6e7], 5 mT at 500 Hz; steady +
5 steps at 2e-5 s), solved by the CPU oracle (C assembly + row-equilibrated
SuperLU with refinement).

Many touching conductors of very different conductivity make this the hard case
for an iterative solver: bodies attached to others through a few edges give
near-null modes of the potential block.  tests/golden/inclusions_32.npz holds, for
the steady state and every step, the three H components on the z-mid slice and
the norms of A, of the H cubes and of the edge current sigma * grad V; and, for
the last step, A itself and the edge current.

Usage:  python tests/golden/make_inclusions.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import qms_oracle as o  # noqa: E402
from alpineqms_gb300 import workloads  # noqa: E402


def main():
    inp, geom = workloads.inclusions_96(seed=2, nt=5, size=32)
    p = dict(xs=inp.xs, ys=inp.ys, zs=inp.zs, dx=inp.dx, dy=inp.dy, dz=inp.dz, dt=inp.dt, Nt=inp.nt, B=inp.B,
             G=inp.G, traj=[(t.v0, t.accel, t.n_accel) for t in inp.traj], props=inp.props_table(),
             excitation=inp.excitation)
    states = o.simulate(p, geom, keep_states=True)
    c = o.materials(inp.xs, inp.ys, inp.zs, geom, inp.props_table())
    oV = o.block_offsets(inp.xs, inp.ys, inp.zs)[3]
    sl = inp.slice_index - 1
    slices, anorm, hnorm, jnorm = [], [], [], []
    for counter, x, H in states:
        cubes = [h.reshape((inp.xs, inp.ys, inp.zs), order="F") for h in H]
        slices.append(np.stack([cb[:, :, sl] for cb in cubes]))
        anorm.append(np.linalg.norm(x[:oV]))
        hnorm.append(np.sqrt(sum(np.dot(h, h) for h in H)))
        jnorm.append(np.linalg.norm(o.edge_current_from_v(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, x)))
    x_last = states[-1][1]
    np.savez_compressed(os.path.join(HERE, "inclusions_32.npz"), slices=np.array(slices), anorm=np.array(anorm),
                        hnorm=np.array(hnorm), jnorm=np.array(jnorm), slice_index=inp.slice_index,
                        a_last=x_last[:oV],
                        j_last=o.edge_current_from_v(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, x_last))
    print("records", len(slices))


if __name__ == "__main__":
    main()
