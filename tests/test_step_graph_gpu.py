"""Whole time steps captured as one CUDA graph, and FGMRES bases longer than one kernel pass.

A chained transient step (same operator as the step before, the field unchanged, the start
residual formed by the step start) runs as one graph: the status reset, the step start with
its rotating history pointers copied in by a graph node, the start residual, and a
conditional WHILE node whose body is a refinement cycle ended by a device-side convergence
test.  On the moving plate the steps after the first few must run that way, converge to the
tolerance, and agree with an FP64 solve of the same step from the same state (tol 1e-14)
within 1e-8 on A and H.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_chained_steps_run_as_one_graph_and_match_fp64():
    from alpineqms_gb300 import workloads
    from alpineqms_gb300.solver import QMSSolver, default_desc
    from alpineqms_gb300.trajectory import VelocitySchedule, scaled_field
    inp, geom = workloads.moving_plate(48, nt=16, plate=(36, 36, 4))
    mk = lambda **kw: QMSSolver(default_desc(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, inp.dt, **kw))
    s = mk()
    s.set_geometry_f64(geom, inp.props_table())
    r64 = mk(precision="fp64", tol=1e-14)
    r64.set_geometry_f64(geom, inp.props_table())
    sched = VelocitySchedule(inp.traj, inp.dt)
    B, G = scaled_field(inp.B, inp.G, inp.excitation, 0.0)
    s.steady(sched.steady(), B, G)
    graphs = 0
    oV = s.n - (inp.xs + 1) * (inp.ys + 1) * (inp.zs + 1)
    for k in range(1, inp.nt + 1):
        v = sched.step(k)
        x_prev = s.get_state()
        st = s.step(v, B, G)
        assert st["status"] == 0 and st["r"] <= 2e-13, (k, st)
        graphs += st["step_graph"]
        if k >= inp.nt - 3:
            r64.set_state(x_prev)
            r64.step(v, B, G)
            assert _rel(s.get_state()[:oV], r64.get_state()[:oV]) <= 1e-8
            h = np.concatenate([q.ravel() for q in s.fields()])
            hd = np.concatenate([q.ravel() for q in r64.fields()])
            assert _rel(h, hd) <= 1e-8
    # the steps after the extrapolation history and the replay count are built up
    assert graphs >= inp.nt - 8, graphs
    s.close()
    r64.close()


def test_long_fgmres_basis_two_passes():
    """FGMRES cycles longer than 32 steps run their Gram-Schmidt and update kernels in two
    passes over the basis; a 48-step basis forced to full length (inner_rtol 1e-30, no graphs)
    reaches the tolerance and agrees with the 32-step solver within 1e-8."""
    from alpineqms_gb300 import workloads
    from alpineqms_gb300.solver import QMSSolver, default_desc
    from alpineqms_gb300.trajectory import VelocitySchedule, scaled_field
    from alpineqms_gb300 import serving
    reqs, _ = serving.poisson_stream(5, 0.05, nt=50)
    inp, geom = reqs[4].inputs, reqs[4].geom           # 48^3, 22 random ellipsoids
    out = {}
    for name, kw in (("m32", {}), ("m48", dict(gmres_m=48, inner_rtol=1e-30, use_graphs=0))):
        s = QMSSolver(default_desc(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, inp.dt, **kw))
        s.set_geometry_f64(geom, inp.props_table())
        sched = VelocitySchedule(inp.traj, inp.dt)
        B, G = scaled_field(inp.B, inp.G, inp.excitation, 0.0)
        s.steady(sched.steady(), B, G)
        for k in (1, 2):
            B, G = scaled_field(inp.B, inp.G, inp.excitation, k * inp.dt)
            st = s.step(sched.step(k), B, G)
            assert st["status"] == 0 and st["r"] <= 2e-13, (name, k, st)
        if name == "m48":
            assert st["inner"] >= 48 * st["outer"] - 1, st     # the cycles ran past 32 steps
        out[name] = s.get_state()
        s.close()
    oV = out["m32"].size - (inp.xs + 1) * (inp.ys + 1) * (inp.zs + 1)
    a, b = out["m48"][:oV], out["m32"][:oV]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-8
