"""Whole time steps captured as one CUDA graph.

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
