"""Parity at the sizes of the workloads themselves.

* The GPU CSR (ia, ja, a, b) bit-identical to the oracle's at 32^3 (the copper
  block) and 96^3 (the 24-ellipsoid inclusion geometry): 2.2 M and 71.6 M
  non-zeros, where 64-bit row pointers and offsets matter (the oracle is
  bit-identical to the reference program, test_oracle_golden.py).
* A seeded 48^3 serving request (22 random ellipsoids, mu_r up to 1e3, touching
  bodies of different sigma) whose first step stalled before the near-null points
  of the potential block's multigrid were taken out: steady state + 3 steps in
  mixed precision, each step's solution checked against the oracle's assembled
  system (scaled FP64 residual of the GPU solution, on the CPU) and against the
  FP64 GPU solver at tol 1e-14 (A, gauge-fixed V, sigma grad V and H within 1e-8).
"""
import numpy as np
import pytest

import qms_oracle as o

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _csr_gpu(s, n, nnz, transient, v, B, G, xp):
    t_ia = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    t_ja = torch.empty(nnz, dtype=torch.int32, device="cuda")
    t_a = torch.empty(nnz, dtype=torch.float64, device="cuda")
    t_b = torch.empty(n, dtype=torch.float64, device="cuda")
    t_x = torch.from_numpy(xp).cuda()
    s.assemble_csr(transient, v, B, G, t_x.data_ptr(), t_ia.data_ptr(), t_ja.data_ptr(), t_a.data_ptr(),
                   t_b.data_ptr())
    torch.cuda.synchronize()
    return t_ia, t_ja, t_a, t_b


@pytest.mark.parametrize("which", ["plain_block_32", "inclusions_96"])
def test_csr_bit_exact_at_workload_size(which):
    from alpineqms_gb300 import workloads
    from alpineqms_gb300.solver import QMSSolver, default_desc
    inp, geom = getattr(workloads, which)()
    xs, ys, zs = inp.xs, inp.ys, inp.zs
    n, nnz, _ = o.sizes(xs, ys, zs)
    rng = np.random.default_rng(7)
    xp = rng.standard_normal(n) * 1e-4
    v, B, G = [-3.0, 0.5, 0.0], np.array(inp.B), np.array([0.01, 0, 0.02, 0, -0.03, 0, 0.02, 0, 0.02])
    c = o.materials(xs, ys, zs, geom, inp.props_table())
    ia, ja, a, b = o.assemble(xs, ys, zs, inp.dx, inp.dy, inp.dz, c, True, inp.dt, v, B, G, xp)
    s = QMSSolver(default_desc(xs, ys, zs, inp.dx, inp.dy, inp.dz, inp.dt))
    s.set_geometry_f64(geom, inp.props_table())
    t_ia, t_ja, t_a, t_b = _csr_gpu(s, n, nnz, True, v, B, G, xp)
    s.close()
    assert np.array_equal(t_ia.cpu().numpy(), ia.astype(np.int64))
    assert int(t_ia[-1].item()) == nnz + 1
    del ia
    assert np.array_equal(t_ja.cpu().numpy(), ja)
    del ja, t_ja
    assert np.array_equal(t_a.cpu().numpy(), a)
    assert np.array_equal(t_b.cpu().numpy(), b)


def test_serving_request_that_stalled_converges_and_matches():
    from alpineqms_gb300 import compare, serving
    from alpineqms_gb300.solver import QMSSolver, default_desc
    from alpineqms_gb300.trajectory import VelocitySchedule, scaled_field
    reqs, _ = serving.poisson_stream(25, 0.05, nt=50)
    inp, geom = reqs[24].inputs, reqs[24].geom
    assert (inp.xs, inp.ys, inp.zs) == (48, 48, 48)
    xs, ys, zs = inp.xs, inp.ys, inp.zs
    n = int(o.sizes(xs, ys, zs)[0])
    c = o.materials(xs, ys, zs, geom, inp.props_table())
    esig = compare.edge_sigma(inp, geom)
    fixer = compare.GaugeFixer(inp, geom, esig)
    s = QMSSolver(default_desc(xs, ys, zs, inp.dx, inp.dy, inp.dz, inp.dt))
    s.set_geometry_f64(geom, inp.props_table())
    r64 = QMSSolver(default_desc(xs, ys, zs, inp.dx, inp.dy, inp.dz, inp.dt, precision="fp64", tol=1e-14))
    r64.set_geometry_f64(geom, inp.props_table())
    sched = VelocitySchedule(inp.traj, inp.dt)
    x_prev = None
    for k in range(4):
        B, G = scaled_field(inp.B, inp.G, inp.excitation, k * inp.dt)
        if k == 0:
            v = sched.steady()
            st = s.steady(v, B, G)
            r64.steady(v, B, G)
        else:
            v = sched.step(k)
            r64.set_state(x_prev)          # the FP64 reference step starts from the same state
            st = s.step(v, B, G)
            r64.step(v, B, G)
        assert st["status"] == 0 and st["r"] <= 2e-13, (k, st)
        x = s.get_state()
        # the oracle's own system for this step (assembled from the GPU's previous state): the
        # scaled FP64 residual of the GPU solution
        ia, ja, a, b = o.assemble(xs, ys, zs, inp.dx, inp.dy, inp.dz, c, k > 0, inp.dt, v, B, G,
                                  x_prev if k > 0 else np.zeros(n))
        M = o.to_scipy(ia, ja, a, n)
        D = np.abs(M.diagonal())
        res = np.linalg.norm((b - M @ x) / D) / np.linalg.norm(x)
        assert res <= 4e-13, (k, res)
        xd = r64.get_state()
        cmp = compare.compare_states(inp, geom, x, xd, s.fields(), r64.fields(), fixer, esig)
        for q in ("A", "V_gauge_fixed", "J", "H"):
            assert cmp[q] <= 1e-8, (k, q, cmp)
        x_prev = x
    s.close()
    r64.close()
