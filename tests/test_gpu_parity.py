"""GPU path vs the CPU oracle, through the C-ABI (libqms_gb300.so).

* K1 CSR assembly: ia/ja/a/b bit-identical to the oracle (which is itself
  bit-identical to the reference program, test_oracle_golden.py).
* K2 matrix-free operator vs the assembled CSR (FP64 to 1e-13, FP32 to 1e-5).
* K7 RHS and K8 H bit-identical to the oracle.
* Whole steady + transient solves vs the oracle's direct solve: rel-L2 <= 1e-8
  for A, H (B/mu) and the edge current sigma*grad V (V itself carries the
  floating constant of isolated conductors, see qms_oracle.DirectSolver).
"""
import os

import numpy as np
import pytest

import qms_oracle as o
from conftest import GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from alpineqms_gb300 import _lib
    _lib.load()


def rel_l2(a, b, floor=0.0):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), floor))


def make_case(xs, ys, zs, seed=0, nmat=3, dxyz=(1e-3, 1.1e-3, 0.9e-3)):
    rng = np.random.default_rng(seed)
    geom = rng.integers(0, nmat + 1, size=(xs, ys, zs)).astype(np.float64)
    props = np.array([[m + 1, *(10 ** rng.uniform(0, 3, 3)), *(10 ** rng.uniform(5, 7.7, 3))] for m in range(nmat)])
    return geom.flatten(order="F"), props, dxyz


def solver_for(xs, ys, zs, d, dt, geom, props, **kw):
    from alpineqms_gb300.solver import QMSSolver, default_desc
    s = QMSSolver(default_desc(xs, ys, zs, *d, dt, **kw))
    s.set_geometry_f64(geom, props)
    return s


CSR_CASES = [
    (6, 7, 8, dict(v=(0.0, 0.0, 0.0), B=(0, 0, 1e-3), G=np.zeros(9))),
    (9, 8, 7, dict(v=(1.5, -0.5, 0.25), B=(2e-3, -1e-3, 5e-3), G=[0.05, 0.02, -0.01, 0.02, -0.03, 0.04, -0.01, 0.04, -0.02])),
    (17, 13, 11, dict(v=(-10.0, 0.0, 2.0), B=(1e-2, 0, 0), G=[0, 0, 0.1, 0, -0.05, 0, 0.1, 0, -0.05])),
]


@pytest.mark.parametrize("xs,ys,zs,par", CSR_CASES)
@pytest.mark.parametrize("transient", [False, True])
def test_csr_assembly_bit_exact(xs, ys, zs, par, transient):
    geom, props, d = make_case(xs, ys, zs, seed=xs)
    dt = 2e-5
    n, nnz, _ = o.sizes(xs, ys, zs)
    rng = np.random.default_rng(1)
    xp = rng.standard_normal(n) * 1e-3
    c = o.materials(xs, ys, zs, geom, props)
    ia, ja, a, b = o.assemble(xs, ys, zs, *d, c, transient, dt, par["v"], par["B"], par["G"], xp)
    s = solver_for(xs, ys, zs, d, dt, geom, props)
    dev = "cuda"
    t_ia = torch.empty(n + 1, dtype=torch.int64, device=dev)
    t_ja = torch.empty(nnz, dtype=torch.int32, device=dev)
    t_a = torch.empty(nnz, dtype=torch.float64, device=dev)
    t_b = torch.empty(n, dtype=torch.float64, device=dev)
    t_x = torch.from_numpy(xp).to(dev)
    s.assemble_csr(transient, par["v"], par["B"], par["G"], t_x.data_ptr(), t_ia.data_ptr(), t_ja.data_ptr(),
                   t_a.data_ptr(), t_b.data_ptr())
    assert np.array_equal(t_ia.cpu().numpy(), ia.astype(np.int64))
    assert np.array_equal(t_ja.cpu().numpy(), ja)
    assert np.array_equal(t_a.cpu().numpy(), a)
    assert np.array_equal(t_b.cpu().numpy(), b)
    s.close()


def test_csr_assembly_golden_inputs():
    """The GPU CSR of the steady system for each golden case equals the reference program's."""
    from alpineqms_gb300.inputs import parse_inputs_text
    for name in GOLDEN_CASES:
        z = load_golden(name)
        inp = parse_inputs_text(bytes(z["inputs_txt"]).decode())
        n = inp.n_dims
        nnz = len(z["ja"])
        v = [t.v0 for t in inp.traj]
        s = solver_for(inp.xs, inp.ys, inp.zs, (inp.dx, inp.dy, inp.dz), inp.dt, z["geom"].flatten(order="F"),
                       inp.props_table())
        t_ia = torch.empty(n + 1, dtype=torch.int64, device="cuda")
        t_ja = torch.empty(nnz, dtype=torch.int32, device="cuda")
        t_a = torch.empty(nnz, dtype=torch.float64, device="cuda")
        t_b = torch.empty(n, dtype=torch.float64, device="cuda")
        s.assemble_csr(False, v, inp.B, inp.G_flat, 0, t_ia.data_ptr(), t_ja.data_ptr(), t_a.data_ptr(),
                       t_b.data_ptr())
        assert np.array_equal(t_ia.cpu().numpy(), z["ia"].astype(np.int64)), name
        assert np.array_equal(t_ja.cpu().numpy(), z["ja"]), name
        assert np.array_equal(t_a.cpu().numpy(), z["a0"]), name
        assert np.array_equal(t_b.cpu().numpy(), z["b0"]), name
        s.close()


@pytest.mark.parametrize("xs,ys,zs,par", CSR_CASES)
@pytest.mark.parametrize("transient", [False, True])
def test_matrix_free_operator_vs_csr(xs, ys, zs, par, transient):
    geom, props, d = make_case(xs, ys, zs, seed=xs + 1)
    dt = 2e-5
    n, nnz, _ = o.sizes(xs, ys, zs)
    c = o.materials(xs, ys, zs, geom, props)
    ia, ja, a, _ = o.assemble(xs, ys, zs, *d, c, transient, dt, par["v"], par["B"], par["G"], np.zeros(n))
    A = o.to_scipy(ia, ja, a, n)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(n) * 1e-3
    yref = A @ x
    s = solver_for(xs, ys, zs, d, dt, geom, props)
    tx = torch.from_numpy(x).cuda()
    ty = torch.empty_like(tx)
    s.apply(transient, par["v"], False, tx.data_ptr(), ty.data_ptr())
    y = ty.cpu().numpy()
    # per-row scale: sum |a_ij x_j| (entries differ from the CSR by a few ulp)
    Aabs = o.to_scipy(ia, ja, np.abs(a), n)
    scale = Aabs @ np.abs(x)
    assert np.max(np.abs(y - yref) / scale) < 1e-13
    tx32 = tx.float()
    ty32 = torch.empty_like(tx32)
    s.apply(transient, par["v"], True, tx32.data_ptr(), ty32.data_ptr())
    assert np.max(np.abs(ty32.cpu().double().numpy() - yref) / scale) < 2e-5
    s.close()


def test_rhs_and_hfield_bit_exact():
    """K7 (via a steady/transient solve's b) and K8 equal the oracle's values for the same x."""
    xs, ys, zs = 10, 9, 11
    geom, props, d = make_case(xs, ys, zs, seed=5)
    dt = 1e-5
    c = o.materials(xs, ys, zs, geom, props)
    n = o.sizes(xs, ys, zs)[0]
    rng = np.random.default_rng(3)
    x = rng.standard_normal(n) * 1e-3
    s = solver_for(xs, ys, zs, d, dt, geom, props)
    s.set_state(x)
    H = s.fields()
    Hr = o.hfield(xs, ys, zs, *d, c, x)
    for q in range(3):
        assert np.array_equal(H[q].ravel(order="F"), Hr[q])
    for ax, idx in (("x", 1), ("x", xs), ("y", 4), ("y", ys), ("z", 1), ("z", 7)):
        sl = s.slices(ax, idx)
        cut = [slice(None)] * 3
        cut["xyz".index(ax)] = idx - 1
        for q in range(3):
            assert np.array_equal(sl[q], H[q][tuple(cut)]), (ax, idx, q)
    s.close()


def _run_gpu(p, geom, precision, steps, **kw):
    from alpineqms_gb300.trajectory import VelocitySchedule, scaled_field
    from alpineqms_gb300.inputs import Trajectory
    traj = [Trajectory(1, *t) for t in p["traj"]]
    sched = VelocitySchedule(traj, p["dt"])
    out = []
    s = solver_for(p["xs"], p["ys"], p["zs"], (p["dx"], p["dy"], p["dz"]), p["dt"], geom, p["props"],
                   precision=precision, **kw)
    B, G = scaled_field(p["B"], p["G"], p.get("excitation"), 0.0)
    st = s.steady(sched.steady(), B, G)
    out.append((s.get_state(), [h.ravel(order="F") for h in s.fields()], st))
    for n in range(1, steps + 1):
        v = sched.step(n)
        B, G = scaled_field(p["B"], p["G"], p.get("excitation"), n * p["dt"])
        st = s.step(v, B, G)
        out.append((s.get_state(), [h.ravel(order="F") for h in s.fields()], st))
    s.close()
    return out


def _conductor_case(moving):
    xs, ys, zs = 16, 14, 12
    geom = np.zeros((xs, ys, zs))
    geom[4:12, 4:10, 4:8] = 1
    geom[6:9, 6:8, 5:7] = 2
    props = np.array([[1, 1, 1, 1, 3.5e7, 3.5e7, 3.5e7], [2, 200, 200, 200, 2e6, 2e6, 2e6]], np.float64)
    traj = [(0.0, -1e6, 1), (0.0, 0.0, 0), (0.0, 0.0, 0)] if moving else [(0.0, 0.0, 0)] * 3
    p = dict(xs=xs, ys=ys, zs=zs, dx=1e-3, dy=1e-3, dz=1e-3, dt=1e-5, Nt=3, B=(1e-3, 2e-3, 1e-2),
             G=np.array([[-0.05, 0, 0], [0, -0.05, 0], [0, 0, 0.1]]), traj=traj, props=props,
             excitation=None if moving else ("cos", 1000.0, 0.0))
    return p, geom.flatten(order="F")


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_harmonic_and_tabulated_motion_vs_direct_oracle(precision):
    """Trajectory types 2 (harmonic, along x) and 3 (a velocity table, along y), which the
    reference stops on (F:135-151): the frame velocity changes every step, and every step's A,
    H and sigma grad V must match the oracle's direct solve with the same velocities to 1e-8."""
    from alpineqms_gb300.inputs import Trajectory
    from alpineqms_gb300.trajectory import VelocitySchedule
    p, geom = _conductor_case(True)
    traj = [Trajectory(2, amp=10.0, freq=1e4, phase=0.5), Trajectory(3, table=(0.0, 3.0, -4.0, 5.0)),
            Trajectory(1, 0.0, 0.0, 0)]
    steps = 5
    sched = VelocitySchedule(traj, p["dt"])
    vel = np.array([sched.steady()] + [sched.step(n) for n in range(1, steps + 1)])
    assert len({tuple(v) for v in vel[1:]}) == steps             # a new operator every step
    ref = o.simulate(dict(p, velocities=vel), geom, steps=steps, keep_states=True)
    s = solver_for(p["xs"], p["ys"], p["zs"], (p["dx"], p["dy"], p["dz"]), p["dt"], geom, p["props"],
                   precision=precision)
    B, G = np.asarray(p["B"], np.float64), np.asarray(p["G"], np.float64).ravel()
    sched = VelocitySchedule(traj, p["dt"])
    c = o.materials(p["xs"], p["ys"], p["zs"], geom, p["props"])
    oV = o.block_offsets(p["xs"], p["ys"], p["zs"])[3]
    for n, (counter, xr, Hr) in enumerate(ref):
        v = sched.steady() if n == 0 else sched.step(n)
        assert np.array_equal(v, vel[n])
        st = s.steady(v, B, G) if n == 0 else s.step(v, B, G)
        assert st["status"] == 0, (n, st)
        x = s.get_state()
        H = [h.ravel(order="F") for h in s.fields()]
        assert rel_l2(x[:oV], xr[:oV]) <= 1e-8, (n, rel_l2(x[:oV], xr[:oV]))
        for q in range(3):
            assert rel_l2(H[q], Hr[q]) <= 1e-8, (n, q)
        jv = o.edge_current_from_v(p["xs"], p["ys"], p["zs"], p["dx"], p["dy"], p["dz"], c, x)
        jr = o.edge_current_from_v(p["xs"], p["ys"], p["zs"], p["dx"], p["dy"], p["dz"], c, xr)
        if np.linalg.norm(jr) > 0:
            assert rel_l2(jv, jr) <= 1e-8, (n, rel_l2(jv, jr))
    s.close()


@pytest.mark.parametrize("moving", [False, True])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("precond", [1, 0], ids=["mg", "jacobi"])
def test_solve_matches_direct_oracle(moving, precision, precond):
    p, geom = _conductor_case(moving)
    ref = o.simulate(p, geom, steps=3, keep_states=True)
    got = _run_gpu(p, geom, precision, 3, precond=precond)
    c = o.materials(p["xs"], p["ys"], p["zs"], geom, p["props"])
    oV = o.block_offsets(p["xs"], p["ys"], p["zs"])[3]
    for (xr_n, (counter, xr, Hr)), (x, H, st) in zip(enumerate(ref), got):
        assert st["status"] == 0
        assert rel_l2(x[:oV], xr[:oV]) <= 1e-8, (counter, rel_l2(x[:oV], xr[:oV]))
        for q in range(3):
            assert rel_l2(H[q], Hr[q]) <= 1e-8, (counter, q)
        jv = o.edge_current_from_v(p["xs"], p["ys"], p["zs"], p["dx"], p["dy"], p["dz"], c, x)
        jr = o.edge_current_from_v(p["xs"], p["ys"], p["zs"], p["dx"], p["dy"], p["dz"], c, xr)
        if np.linalg.norm(jr) > 0:
            assert rel_l2(jv, jr) <= 1e-8, (counter, rel_l2(jv, jr))


def test_bad_material_id_rejected():
    from alpineqms_gb300._lib import QMSError
    xs = ys = zs = 6
    geom = np.zeros(xs * ys * zs)
    geom[5] = 7.0
    props = np.array([[1, 1, 1, 1, 0, 0, 0]], np.float64)
    from alpineqms_gb300.solver import QMSSolver, default_desc
    with QMSSolver(default_desc(xs, ys, zs, 1e-3, 1e-3, 1e-3, 1e-5)) as s:
        with pytest.raises(QMSError):
            s.set_geometry_f64(geom, props)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_dropin_dumps_vs_reference_program(name, tmp_path):
    """The drop-in QMS_3D run on each golden case writes the same dump files (record
    structure identical, values within 1e-8 relative L2 of the reference program's)."""
    from alpineqms_gb300 import qms3d
    from alpineqms_gb300.records import read_records
    z = load_golden(name)
    (tmp_path / "inputs.txt").write_bytes(bytes(z["inputs_txt"]))
    z["geom"].astype("<f8").flatten(order="F").tofile(str(tmp_path / "geom.bin"))
    qms3d.run(str(tmp_path / "inputs.txt"), workdir=str(tmp_path), log=lambda *a: None)
    for group in (("Hx.bin", "Hy.bin", "Hz.bin"), ("Hx_all.bin", "Hy_all.bin", "Hz_all.bin")):
        keys = ["dump_" + nm.replace(".", "_") for nm in group]
        if keys[0] not in z:
            for nm in group:
                assert not (tmp_path / nm).exists(), nm
            continue
        got, ref = [], []
        for nm, key in zip(group, keys):
            data = (tmp_path / nm).read_bytes()
            assert len(data) == len(bytes(z[key])), nm           # same record structure
            (tmp_path / ("ref_" + nm)).write_bytes(bytes(z[key]))
            got.append(read_records(str(tmp_path / nm)))
            ref.append(read_records(str(tmp_path / ("ref_" + nm))))
        # compare the three components of each record together: a component that is
        # identically zero in the exact solution (e.g. Hx under a uniform Bz) holds only
        # round-off in both runs
        for rec in range(len(ref[0])):
            a = np.concatenate([got[q][rec] for q in range(3)])
            b = np.concatenate([ref[q][rec] for q in range(3)])
            assert rel_l2(a, b, floor=1e-30) <= 1e-8, (group[0], rec, rel_l2(a, b))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_plain_block_32_twenty_steps(precision):
    """The 32^3 copper block under a 1 kHz field (steady + 20 steps): every z-mid H
    slice record, and the whole A block, edge current sigma grad V and H cubes at the
    fixture's full steps, within 1e-8 relative L2 of the oracle's direct solve
    (tests/golden/plain_block_32.npz, made by tests/golden/make_config1.py)."""
    from alpineqms_gb300 import workloads
    from alpineqms_gb300.trajectory import VelocitySchedule, scaled_field
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "plain_block_32.npz"))
    inp, geom = workloads.plain_block_32()
    sched = VelocitySchedule(inp.traj, inp.dt)
    s = solver_for(inp.xs, inp.ys, inp.zs, (inp.dx, inp.dy, inp.dz), inp.dt, geom, inp.props_table(),
                   precision=precision)
    sl = int(z["slice_index"]) - 1
    for n in range(0, inp.nt + 1):
        B, G = scaled_field(inp.B, inp.G, inp.excitation, n * inp.dt)
        st = s.steady(sched.steady(), B, G) if n == 0 else s.step(sched.step(n), B, G)
        assert st["status"] == 0, (n, st)
        H = s.fields()
        got = np.stack([h.reshape((inp.xs, inp.ys, inp.zs), order="F")[:, :, sl] for h in H])
        assert rel_l2(got, z["slices"][n]) <= 1e-8, (n, rel_l2(got, z["slices"][n]))
        hn = np.sqrt(sum(np.dot(h.ravel(), h.ravel()) for h in H))
        assert abs(hn - z["hnorm"][n]) <= 1e-8 * z["hnorm"][n], (n, hn, z["hnorm"][n])
        x = s.get_state()
        xa = x[:o.block_offsets(inp.xs, inp.ys, inp.zs)[3]]
        assert abs(np.linalg.norm(xa) - z["anorm"][n]) <= 1e-8 * z["anorm"][n]
        if n in set(int(q) for q in z["full_steps"]):
            # whole vectors at these steps: A, the edge current sigma grad V and the H cubes
            c = o.materials(inp.xs, inp.ys, inp.zs, geom, inp.props_table())
            j = o.edge_current_from_v(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, x)
            assert rel_l2(xa, z["a_%d" % n]) <= 1e-8, (n, rel_l2(xa, z["a_%d" % n]))
            assert rel_l2(j, z["j_%d" % n]) <= 1e-8, (n, rel_l2(j, z["j_%d" % n]))
            h = np.concatenate([q.ravel(order="F") for q in H])
            assert rel_l2(h, z["h_%d" % n]) <= 1e-8, (n, rel_l2(h, z["h_%d" % n]))
    s.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_random_inclusions_32_vs_oracle(precision):
    """24 random ellipsoids (mu_r up to 1e3, sigma 1e5..6e7) at 32^3, steady + 5 steps: every
    z-mid H slice, the A and H norms and the edge-current norm within 1e-8 of the oracle's
    direct solve, and the final A and sigma * grad V within 1e-8 (tests/golden/inclusions_32.npz,
    made by tests/golden/make_inclusions.py).  Bodies attached to others through a few edges
    make this the hard case for the potential block."""
    from alpineqms_gb300 import workloads
    from alpineqms_gb300.trajectory import VelocitySchedule, scaled_field
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "inclusions_32.npz"))
    inp, geom = workloads.inclusions_96(seed=2, nt=5, size=32)
    c = o.materials(inp.xs, inp.ys, inp.zs, geom, inp.props_table())
    oV = o.block_offsets(inp.xs, inp.ys, inp.zs)[3]
    sched = VelocitySchedule(inp.traj, inp.dt)
    s = solver_for(inp.xs, inp.ys, inp.zs, (inp.dx, inp.dy, inp.dz), inp.dt, geom, inp.props_table(),
                   precision=precision)
    sl = int(z["slice_index"]) - 1
    for n in range(0, inp.nt + 1):
        B, G = scaled_field(inp.B, inp.G, inp.excitation, n * inp.dt)
        st = s.steady(sched.steady(), B, G) if n == 0 else s.step(sched.step(n), B, G)
        assert st["status"] == 0, (n, st)
        H = s.fields()
        got = np.stack([h.reshape((inp.xs, inp.ys, inp.zs), order="F")[:, :, sl] for h in H])
        assert rel_l2(got, z["slices"][n]) <= 1e-8, (n, rel_l2(got, z["slices"][n]))
        hn = np.sqrt(sum(np.dot(h.ravel(), h.ravel()) for h in H))
        assert abs(hn - z["hnorm"][n]) <= 1e-8 * z["hnorm"][n], (n, hn, z["hnorm"][n])
        x = s.get_state()
        assert abs(np.linalg.norm(x[:oV]) - z["anorm"][n]) <= 1e-8 * z["anorm"][n]
        jn = np.linalg.norm(o.edge_current_from_v(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, x))
        assert abs(jn - z["jnorm"][n]) <= 1e-8 * max(z["jnorm"][n], 1e-300) + 1e-300, (n, jn, z["jnorm"][n])
    assert rel_l2(x[:oV], z["a_last"]) <= 1e-8, rel_l2(x[:oV], z["a_last"])
    j = o.edge_current_from_v(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, c, x)
    assert rel_l2(j, z["j_last"]) <= 1e-8, rel_l2(j, z["j_last"])
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [dict(mg_coupling=0), dict(mg_coupling=1, mg_alpha=1.0),
                                     dict(mg_coupling=1, mg_coarse_sweeps=2, mg_sweeps=2, mg_omega=0.8)],
                         ids=["block-diagonal", "triangular-alpha1", "triangular-2sweeps"])
def test_preconditioner_variants_match_direct_oracle(variant):
    """The block-diagonal and lower block-triangular multigrid, with and without the
    over-corrected coarse grid, all converge to the direct solution of the moving conductor."""
    p, geom = _conductor_case(True)
    ref = o.simulate(p, geom, steps=3, keep_states=True)
    got = _run_gpu(p, geom, "mixed", 3, **variant)
    oV = o.block_offsets(p["xs"], p["ys"], p["zs"])[3]
    for (counter, xr, Hr), (x, H, st) in zip(ref, got):
        assert st["status"] == 0
        assert rel_l2(x[:oV], xr[:oV]) <= 1e-8, (counter, variant)
        for q in range(3):
            assert rel_l2(H[q], Hr[q]) <= 1e-8, (counter, q, variant)


@pytest.mark.gpu
def test_double_float_residual_agrees_with_fp64():
    """The refinement's residual after the first iteration of a solve is evaluated in
    double-float from an FP64 anchor; at the converged state it must agree with the exact FP64
    residual of the same state (qms_residual_norm) to a few 1e-15 of |x|."""
    p, geom = _conductor_case(True)
    from alpineqms_gb300.trajectory import VelocitySchedule, scaled_field
    from alpineqms_gb300.inputs import Trajectory
    sched = VelocitySchedule([Trajectory(1, *t) for t in p["traj"]], p["dt"])
    s = solver_for(p["xs"], p["ys"], p["zs"], (p["dx"], p["dy"], p["dz"]), p["dt"], geom, p["props"],
                   precision="mixed")
    B, G = scaled_field(p["B"], p["G"], p.get("excitation"), 0.0)
    s.steady(sched.steady(), B, G)
    for n in range(1, 5):
        v = sched.step(n)
        B, G = scaled_field(p["B"], p["G"], p.get("excitation"), n * p["dt"])
        st = s.step(v, B, G)
        exact = s.residual_norm(True, v)
        assert st["outer"] >= 1                      # at least one double-float residual was used
        assert abs(st["r"] - exact) <= 0.25 * exact + 5e-15, (n, st["r"], exact)
    s.close()


@pytest.mark.gpu
def test_chained_residual_does_not_drift():
    """A transient run chains each step's anchor to the previous step's final double-float
    residual for up to 32 steps.  Over 40 steps with one operator (a full chain, a re-anchor and
    the start of the next chain) every step's final residual must agree with the exact FP64
    residual of the returned state to a tenth of the tolerance."""
    p, geom = _conductor_case(True)
    from alpineqms_gb300.trajectory import VelocitySchedule
    from alpineqms_gb300.inputs import Trajectory
    sched = VelocitySchedule([Trajectory(1, *t) for t in p["traj"]], p["dt"])
    s = solver_for(p["xs"], p["ys"], p["zs"], (p["dx"], p["dy"], p["dz"]), p["dt"], geom, p["props"],
                   precision="mixed")
    tol = s.desc.tol
    B, G = np.asarray(p["B"], np.float64), np.asarray(p["G"], np.float64).ravel()
    s.steady(sched.steady(), B, G)
    v = sched.step(1)
    worst = 0.0
    for n in range(1, 41):
        st = s.step(v, B, G)
        assert st["status"] == 0, (n, st)
        exact = s.residual_norm(True, v)
        assert exact <= tol * 1.5, (n, exact)
        worst = max(worst, abs(st["r"] - exact))
    s.close()
    assert worst <= 0.1 * tol, worst


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2, 3])
def test_extrapolated_start_residual_by_linearity(order):
    """Once three steps in a row are chained, the residual of the extrapolated start follows from
    the anchor and the stored differences D^-1 M (x_n - x_(n-1)) of the last steps, without a
    stencil pass, and the anchor takes b - b_prev from x_n - x_(n-1) (qk_step_start).  At the
    last step the start residual must equal the exact FP64 residual of the same start state
    (rebuilt here from the returned solutions), the right-hand side formed on demand must equal
    the oracle's, and every step must reach the tolerance with a final residual that agrees with
    the exact one."""
    p, geom = _conductor_case(True)
    from alpineqms_gb300.trajectory import VelocitySchedule
    from alpineqms_gb300.inputs import Trajectory
    sched = VelocitySchedule([Trajectory(1, *t) for t in p["traj"]], p["dt"])
    s = solver_for(p["xs"], p["ys"], p["zs"], (p["dx"], p["dy"], p["dz"]), p["dt"], geom, p["props"],
                   precision="mixed", extrapolate=order, start_ls=0)
    B, G = np.asarray(p["B"], np.float64), np.asarray(p["G"], np.float64).ravel()
    s.steady(sched.steady(), B, G)
    v = sched.step(1)                    # one constant frame velocity: every step has the same operator
    X = []
    for n in range(1, 8):
        st = s.step(v, B, G)
        assert st["status"] == 0, (n, st)
        exact = s.residual_norm(True, v)
        assert abs(st["r"] - exact) <= 0.25 * exact + 5e-15, (n, st["r"], exact)
        X.append(s.get_state())
    # the start of the last step: the solutions before it, extrapolated
    if order == 1:
        x_start = 2.0 * X[-2] - X[-3]
    elif order == 2:
        x_start = 3.0 * (X[-2] - X[-3]) + X[-4]
    else:
        x_start = 4.0 * (X[-2] + X[-4]) - 6.0 * X[-3] - X[-5]
    # the chained steps took b - b_prev from the state difference: the last step's b, formed on
    # demand from its start state, is still the reference's right-hand side bit for bit
    c = o.materials(p["xs"], p["ys"], p["zs"], geom, p["props"])
    _, _, _, br = o.assemble(p["xs"], p["ys"], p["zs"], p["dx"], p["dy"], p["dz"], c, True, p["dt"], v, B, G,
                             x_prev=X[-2])
    assert np.array_equal(s.get_rhs(), br)
    s.set_state(x_start)                 # b is still the last step's
    exact0 = s.residual_norm(True, v)
    s.close()
    assert exact0 > 0
    assert abs(st["r0"] - exact0) <= 1e-3 * exact0 + 1e-15, (st["r0"], exact0)


@pytest.mark.gpu
@pytest.mark.parametrize("nls", [1, 2, 4])
def test_least_squares_start(nls):
    """With the least-squares start the first residual of a chained step is that of x_n plus the
    reported combination of the last state differences: it must equal the exact FP64 residual of
    that start state (rebuilt here from the returned solutions), be no larger than the residual
    of the polynomial start of the same history, and every step must reach the tolerance with a
    final residual that agrees with the exact one."""
    p, geom = _conductor_case(True)
    from alpineqms_gb300.trajectory import VelocitySchedule
    from alpineqms_gb300.inputs import Trajectory
    sched = VelocitySchedule([Trajectory(1, *t) for t in p["traj"]], p["dt"])
    s = solver_for(p["xs"], p["ys"], p["zs"], (p["dx"], p["dy"], p["dz"]), p["dt"], geom, p["props"],
                   precision="mixed", start_ls=nls)
    B, G = np.asarray(p["B"], np.float64), np.asarray(p["G"], np.float64).ravel()
    s.steady(sched.steady(), B, G)
    v = sched.step(1)
    X, S = [], []
    for n in range(1, 11):
        st = s.step(v, B, G)
        assert st["status"] == 0, (n, st)
        exact = s.residual_norm(True, v)
        assert abs(st["r"] - exact) <= 0.25 * exact + 5e-15, (n, st["r"], exact)
        X.append(s.get_state())
        S.append(st)
    st = S[-1]
    assert st["start_ls"] == nls, st
    gam = st["start_coef"]
    assert all(np.isfinite(gam)) and all(gam[j] == 0.0 for j in range(nls, 4)), gam
    # the start of the last step, rebuilt: x_n = X[-2], the differences before it
    x_start = X[-2].copy()
    for j in range(nls):
        x_start += gam[j] * (X[-2 - j] - X[-3 - j])
    cubic = 4.0 * (X[-2] + X[-4]) - 6.0 * X[-3] - X[-5]
    s.set_state(x_start)                 # b is still the last step's
    exact0 = s.residual_norm(True, v)
    s.set_state(cubic)
    exact_cubic = s.residual_norm(True, v)
    s.close()
    assert abs(st["r0"] - exact0) <= 1e-3 * exact0 + 1e-15, (st["r0"], exact0)
    if nls >= 3:
        assert exact0 <= 1.01 * exact_cubic, (exact0, exact_cubic)
    assert st["start_pred"] <= 1.001 * st["start_base"], st


@pytest.mark.gpu
@pytest.mark.parametrize("xs,ys,zs,dt,seed", [(10, 9, 11, 1e-5, 5), (26, 24, 22, 2.7e-5, 11)])
def test_transient_rhs_bit_exact(xs, ys, zs, dt, seed):
    """The solver's transient right-hand side (K7 with the per-geometry edge sigma and sigma / dt
    stored once, the divisions by dt h through a corrected reciprocal) equals the oracle's
    assembled RHS bit for bit."""
    geom, props, d = make_case(xs, ys, zs, seed=seed)
    c = o.materials(xs, ys, zs, geom, props)
    n = o.sizes(xs, ys, zs)[0]
    x = np.random.default_rng(7 + seed).standard_normal(n) * 1e-3
    v, B = (1.5, -0.5, 0.25), (2e-3, -1e-3, 5e-3)
    G = np.array([0.05, 0.02, -0.01, 0.02, -0.03, 0.04, -0.01, 0.04, -0.02])
    s = solver_for(xs, ys, zs, d, dt, geom, props)
    s.set_state(x)
    s.step(v, B, G)
    b = s.get_rhs()
    s.close()
    _, _, _, br = o.assemble(xs, ys, zs, *d, c, True, dt, v, B, G, x_prev=x)
    assert np.array_equal(b, br)
