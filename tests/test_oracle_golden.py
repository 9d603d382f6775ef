"""The CPU oracle against fixtures produced by executing the reference itself.

tests/golden/*.npz were written by tests/golden/make_golden.py, which runs
3D/QMS_3D.f90 through a Fortran-subset interpreter with SuperLU in place of
PARDISO and records every CSR matrix, right-hand side and solution the
program produced, plus its H dump files.  Here the C restatement
(oracle/qms_oracle.c) must reproduce all of them bit for bit.
"""
import io
import os
import tempfile

import numpy as np
import pytest

import qms_oracle as o
from alpineqms_gb300.inputs import parse_inputs_text
from alpineqms_gb300.records import DumpWriter, read_records, slice_of
from conftest import GOLDEN_CASES, load_golden


def replay(z):
    """Yield (call index, ia, ja, a, b) from the oracle for each solver call of the golden run."""
    inp = parse_inputs_text(bytes(z["inputs_txt"]).decode())
    c = o.materials(inp.xs, inp.ys, inp.zs, z["geom"].flatten(order="F"), inp.props_table())
    v = np.array([o.trajectory(t.v0, t.accel, t.n_accel, 0, inp.dt) for t in inp.traj])
    acc = [0.0, 0.0, 0.0]
    out = []
    for q, ph in enumerate(z["phases"]):
        if ph == -1:
            continue
        if q == 0:
            csr = o.assemble(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, False, inp.dt, v, inp.B, inp.G_flat)
        else:
            nv = []
            for d, t in enumerate(inp.traj):
                vv, acc[d] = o.step_velocity(t.v0, t.accel, t.n_accel, q, inp.dt, v[d], acc[d])
                nv.append(vv)
            v = np.array(nv)
            csr = o.assemble(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, True, inp.dt, v, inp.B,
                             inp.G_flat, z[f"x{q - 1}"])
        out.append((q, *csr))
    return inp, c, out


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_csr_bit_exact_vs_reference_program(name):
    z = load_golden(name)
    _, _, calls = replay(z)
    assert len(calls) >= 3
    for q, ia, ja, a, b in calls:
        assert np.array_equal(ia, z["ia"]), f"call {q}: ia"
        assert np.array_equal(ja, z["ja"]), f"call {q}: ja"
        assert np.array_equal(a, z[f"a{q}"]), f"call {q}: a_mat"
        assert np.array_equal(b, z[f"b{q}"]), f"call {q}: b_vec"


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_dumps_bit_exact_vs_reference_program(name):
    """Oracle H (from the reference's own solutions) through the product dump writer."""
    z = load_golden(name)
    inp = parse_inputs_text(bytes(z["inputs_txt"]).decode())
    c = o.materials(inp.xs, inp.ys, inp.zs, z["geom"].flatten(order="F"), inp.props_table())
    with tempfile.TemporaryDirectory() as td:
        w = DumpWriter(inp, td)
        for q, ph in enumerate(z["phases"]):
            if ph == -1:
                continue
            H = [h.reshape((inp.xs, inp.ys, inp.zs), order="F")
                 for h in o.hfield(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, z[f"x{q}"])]
            if w.wants_slice(q):
                w.write_slice([slice_of(h, inp.slice_axis, inp.slice_index) for h in H])
            w.write_cube(H)
        w.close()
        for nm in ("Hx.bin", "Hy.bin", "Hz.bin", "Hx_all.bin", "Hy_all.bin", "Hz_all.bin"):
            key = "dump_" + nm.replace(".", "_")
            path = os.path.join(td, nm)
            if key in z:
                got = open(path, "rb").read()
                assert got == bytes(z[key]), nm
            else:
                assert not os.path.exists(path), nm


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_simulate_matches_reference_solutions(name):
    """Full oracle run (materials, trajectory, assembly, SuperLU) vs the reference program's x."""
    z = load_golden(name)
    inp = parse_inputs_text(bytes(z["inputs_txt"]).decode())
    p = dict(xs=inp.xs, ys=inp.ys, zs=inp.zs, dx=inp.dx, dy=inp.dy, dz=inp.dz, dt=inp.dt, Nt=inp.nt,
             B=inp.B, G=inp.G, traj=[(t.v0, t.accel, t.n_accel) for t in inp.traj], props=inp.props_table())
    geom = z["geom"].flatten(order="F")
    states = o.simulate(p, geom, keep_states=True)
    c = o.materials(inp.xs, inp.ys, inp.zs, geom, inp.props_table())
    oV = o.block_offsets(inp.xs, inp.ys, inp.zs)[3]
    for (counter, x, _H) in states:
        ref = z[f"x{counter}"]
        assert rel_l2(x[:oV], ref[:oV]) <= 1e-12
        jv = o.edge_current_from_v(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, x)
        jr = o.edge_current_from_v(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, ref)
        assert rel_l2(jv, jr, floor=current_scale(inp, c, ref, oV)) <= 1e-10


def current_scale(inp, c, x, oV):
    """Eddy-current scale sigma * |A| / dt: the floor for relative errors of sigma grad V
    (which vanishes when nothing varies in time)."""
    return float(np.max(c["sig_x"]) * np.linalg.norm(x[:oV]) / inp.dt * 1e-6)


def rel_l2(a, b, floor=0.0):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), floor))


def test_sizes_match_closed_forms():
    # n_dims (F:175) and nnz from the row predicates
    assert o.sizes(32, 32, 32)[:2] == (140481, 2229525)
    assert o.sizes(96, 96, 96)[:2] == (3622465, 71603605)
    assert o.sizes(128, 64, 32)[:2] == (1092033, 19874837)
    n, nnz, ex = o.sizes(101, 101, 101)
    assert nnz > ex          # first cubic size whose true nnz exceeds the reference's guard


def _uniform_case(xs=10, ys=11, zs=12, B=(3e-3, -2e-3, 5e-3)):
    return dict(xs=xs, ys=ys, zs=zs, dx=1e-3, dy=1.2e-3, dz=0.9e-3, dt=1e-5, Nt=2, B=B, G=np.zeros((3, 3)),
                traj=[(0.0, 0.0, 0)] * 3, props=np.array([[1, 1, 1, 1, 0, 0, 0]], np.float64))


def test_known_answer_uniform_field():
    """sigma = 0, mu_r = 1, no gradient, v = 0: A = B x r / 2 is in the kernel of the
    operator, so the steady solve gives H = B_in / mu0 in every cell (F:460-469, F:1346-1376).
    The tolerance is the direct solver's round-off: the matrix rows span ~18 decades
    (air V rows ~1e-6, A rows ~1e12), and SuperLU lands within a few 1e-9 of the exact answer."""
    p = _uniform_case()
    geom = np.zeros(p["xs"] * p["ys"] * p["zs"])
    states = o.simulate(p, geom, steps=0, keep_states=True)
    _, _, H = states[0]
    for h, bc in zip(H, p["B"]):
        assert np.allclose(h, bc / o.MU0, rtol=2e-8)


def test_known_answer_static_fixed_point():
    """Static excitation and v = 0 with a conductor: the steady state is a fixed point of
    the backward-Euler step (F:1475, F:1925-1928)."""
    p = _uniform_case()
    p["props"] = np.array([[1, 1, 1, 1, 5.8e7, 5.8e7, 5.8e7], [2, 30, 30, 30, 0, 0, 0]], np.float64)
    geom = np.zeros((p["xs"], p["ys"], p["zs"]))
    geom[3:7, 3:8, 4:8] = 1
    geom[5:7, 5:7, 5:7] = 2
    states = o.simulate(p, geom.flatten(order="F"), steps=2, keep_states=True)
    x0, H0 = states[0][1], states[0][2]
    c = o.materials(p["xs"], p["ys"], p["zs"], geom.flatten(order="F"), p["props"])
    oV = o.block_offsets(p["xs"], p["ys"], p["zs"])[3]
    for _, x, H in states[1:]:
        assert rel_l2(x[:oV], x0[:oV]) <= 1e-10
        for h, h0 in zip(H, H0):
            assert rel_l2(h, h0) <= 1e-10
        jv = o.edge_current_from_v(p["xs"], p["ys"], p["zs"], p["dx"], p["dy"], p["dz"], c, x)
        # V = 0 up to the conductor's floating constant: no current from grad V
        assert np.abs(jv).max() <= 1e-9 * (p["props"][0, 4] * np.abs(x0[:oV]).max() / p["dt"]) * p["dx"]
