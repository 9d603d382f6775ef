"""CPU checks of alpineqms_gb300.compare: the gauge-fixed comparison of V.

A conductor that no conducting path links to the Dirichlet shell has a
potential pinned only by the 1e-12 S/m floor (3D/QMS_3D.f90:1236-1285), so a
constant on it is (to ~19 decades) a null mode of the system.  Shifting V by a
constant on such a body must leave the gauge-fixed V, the edge current and A
unchanged; shifting the interior of a body that touches the shell must not."""
import numpy as np

import qms_oracle as o
from alpineqms_gb300 import compare
from alpineqms_gb300.inputs import Material, QMSInputs, Trajectory


def _case():
    xs, ys, zs = 14, 12, 10
    geom = np.zeros((xs, ys, zs))
    geom[3:7, 3:7, 3:6] = 1          # floating copper block
    geom[8:11, 4:8, 3:7] = 2         # floating steel block (touches nothing)
    geom[0:5, 9:11, 2:8] = 1         # a bar reaching the Dirichlet shell: grounded
    mats = [Material(1.0, (1.0, 1.0, 1.0), (5.8e7,) * 3), Material(2.0, (100.0,) * 3, (2e6,) * 3)]
    inp = QMSInputs(xs, ys, zs, 1e-3, 1e-3, 1e-3, 1e-5, 1, 1, "z", 5, "no", (1e-3, 2e-3, 5e-3),
                    ((0, 0, 0),) * 3, tuple(Trajectory(1, 0.0, 0.0, 0) for _ in range(3)), mats, "geom.bin")
    return inp, geom.flatten(order="F")


def _solve(inp, geom):
    c = o.materials(inp.xs, inp.ys, inp.zs, geom, inp.props_table())
    B = np.array(inp.B)
    ia, ja, a, b = o.assemble(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, False, inp.dt,
                              np.array([-2.0, 0.0, 0.0]), B, np.zeros(9))
    ds = o.DirectSolver()
    ds.factor(ia, ja, a, len(b))
    return ds.solve(b)


def test_bodies_found():
    inp, geom = _case()
    f = compare.GaugeFixer(inp, geom)
    # three connected conducting bodies: two floating blocks and the grounded bar
    assert f.floating.sum() == 2 and (~f.floating).sum() == 1


def test_floating_constant_is_ignored_and_grounded_one_is_not():
    inp, geom = _case()
    x = _solve(inp, geom)
    f = compare.GaugeFixer(inp, geom)
    Nx, Ny, Nz = inp.xs + 1, inp.ys + 1, inp.zs + 1
    oV = len(x) - Nx * Ny * Nz
    for comp in np.unique(f.labels):
        xs = x.copy()
        nodes = f.nodes[f.labels == comp]
        # the Dirichlet values stay put (F:393-396): only the interior nodes of a body move
        i, rest = nodes % Nx, nodes // Nx
        j, k = rest % Ny, rest // Ny
        nodes = nodes[~((i <= 1) | (i >= Nx - 2) | (j <= 1) | (j >= Ny - 2) | (k <= 1) | (k >= Nz - 2))]
        xs[oV + nodes] += 0.37 * (1.0 + np.abs(x[oV:]).max())
        r = compare.compare_states(inp, geom, xs, x, fixer=f)
        assert r["A"] == 0.0
        assert r["V_raw"] > 1e-3
        if f.floating[comp]:
            assert r["V_gauge_fixed"] <= 1e-11, r      # rounding of a shift ~1e3 x |V|
            assert r["J"] <= 1e-11, r
        else:
            assert r["V_gauge_fixed"] > 1e-3, r
            assert r["J"] > 1e-6, r


def test_identical_states_compare_to_zero():
    inp, geom = _case()
    x = _solve(inp, geom)
    r = compare.compare_states(inp, geom, x, x.copy())
    assert all(v == 0.0 for v in r.values())
