"""The host-side velocity and excitation schedule against the oracle's restatement of the
reference's trajectory_1 and the first-step acceleration pad (3D/QMS_3D.f90:1428-1449,
2331-2350), bit for bit."""
import numpy as np
import pytest

import qms_oracle as o
from alpineqms_gb300.inputs import Trajectory
from alpineqms_gb300.trajectory import VelocitySchedule, excitation_scale, scaled_field, trajectory_1

TRAJS = [
    [(0.0, -1e6, 1), (0.0, 0.0, 0), (0.0, 0.0, 0)],        # a ramp in the first step (the bench plate)
    [(2.5, 0.0, 0), (-1.0, 0.0, 0), (0.0, 3.0, 7)],         # constant velocities: the pad applies
    [(1e-3, 5e2, 4), (0.0, -2e3, 12), (7.0, 1e-9, 3)],
]


@pytest.mark.parametrize("traj", TRAJS)
def test_schedule_matches_oracle(traj):
    dt = 1e-5
    sched = VelocitySchedule([Trajectory(1, *t) for t in traj], dt)
    prev = [o.trajectory(v0, a, n, 0, dt) for (v0, a, n) in traj]
    assert sched.steady() == prev
    acc = [0.0, 0.0, 0.0]
    for counter in range(1, 21):
        got = sched.step(counter)
        for d, (v0, a, n) in enumerate(traj):
            v, acc[d] = o.step_velocity(v0, a, n, counter, dt, prev[d], acc[d])
            assert got[d] == v, (counter, d, got[d], v)
            prev[d] = v


def test_trajectory_1_matches_oracle():
    for (v0, a, t) in [(0.0, -1e6, 1), (3.0, 2.0, 5), (-1.0, 0.5, 0)]:
        for n in range(0, 9):
            assert trajectory_1(v0, a, t, n, 1e-5) == o.trajectory(v0, a, t, n, 1e-5)


def test_excitation():
    for exc in [None, ("cos", 1000.0, 0.0), ("sin", 50.0, 0.3)]:
        for t in [0.0, 1e-5, 3.7e-4]:
            assert excitation_scale(exc, t) == o.excitation_scale(exc, t)
    B, G = (1e-3, 2e-3, 1e-2), np.arange(9.0)
    b0, g0 = scaled_field(B, G, None, 1.0)
    assert np.array_equal(b0, B) and np.array_equal(g0, G)   # exact copies without excitation
    b1, g1 = scaled_field(B, G, ("cos", 1000.0, 0.0), 2.5e-4)
    s = excitation_scale(("cos", 1000.0, 0.0), 2.5e-4)
    assert np.array_equal(b1, np.asarray(B) * s) and np.array_equal(g1, G * s)


MIXED = [Trajectory(2, amp=0.75, freq=2500.0, phase=0.3),      # harmonic
         Trajectory(3, table=(0.0, 1.5, -2.0, 4.0)),             # a table, held after its end
         Trajectory(1, 2.5, 0.0, 3)]                              # type 1 with the pad


def test_schedule_types_two_and_three():
    """Harmonic and tabulated axes follow their formulas; only the type-1 axis gets the
    first-step pad, and it gets the same pad as in a pure type-1 schedule."""
    import math
    dt = 1e-5
    sched = VelocitySchedule(MIXED, dt)
    pure = VelocitySchedule([Trajectory(1, 2.5, 0.0, 3)] * 3, dt)
    v = [sched.steady()] + [sched.step(n) for n in range(1, 9)]
    w = [pure.steady()] + [pure.step(n) for n in range(1, 9)]
    for n in range(9):
        assert v[n][0] == 0.75 * math.sin(2.0 * math.pi * 2500.0 * (n * dt) + 0.3)
        assert v[n][1] == (0.0, 1.5, -2.0, 4.0)[min(n, 3)]
        assert v[n][2] == w[n][2]
    assert v[1][2] != v[0][2]                                    # the pad moved the first step


@pytest.mark.parametrize("traj", [MIXED, [Trajectory(1, *t) for t in TRAJS[2]]])
def test_server_schedule_matches_python(traj):
    """The native server's schedule (qms_srv_velocities, host only) equals the drop-in's."""
    import ctypes
    from alpineqms_gb300 import _lib, build as b
    from alpineqms_gb300.inputs import parse_inputs_text
    from alpineqms_gb300.serving import request_struct
    from alpineqms_gb300.workloads import inputs_text, plain_block_32
    b.build()
    L = _lib.load()
    inp, _ = plain_block_32(nt=12)
    inp.traj = tuple(traj)
    inp = parse_inputs_text(inputs_text(inp))                  # through the file grammar
    r, keep = request_struct(inp, None, False, 0)
    nsteps = 12
    out = np.zeros((nsteps + 1, 3))
    assert L.qms_srv_velocities(ctypes.byref(r), nsteps, out.ctypes.data) == 0
    sched = VelocitySchedule(inp.traj, inp.dt)
    want = np.array([sched.steady()] + [sched.step(n) for n in range(1, nsteps + 1)])
    assert np.array_equal(out, want), np.abs(out - want).max()
    bad, keep2 = request_struct(inp, None, False, 0)
    bad.traj_kind[1] = 3
    bad.traj_len[1] = 0
    assert L.qms_srv_velocities(ctypes.byref(bad), nsteps, out.ctypes.data) == -1     # QMS_ERR_ARG
