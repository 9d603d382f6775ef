"""Frame velocity and excitation schedule of a run (host-side scalars).

trajectory_1 (3D/QMS_3D.f90:2331-2350): v(n) = v0 + a*n*dt while n <= t,
v0 + a*t*dt afterwards.  The first transient step adds a small acceleration
"pad" when a*dt < v0*1E-8 (F:1428-1449); 1E-8 is a default-real (single
precision) literal and the pad state is static storage that starts at zero.
The same velocity drives the steady state (n = 0, F:431-433).

The optional excitation scales the whole background field (B_in and its
gradient) by s(t) at t = n*dt.
"""
from __future__ import annotations

import math

import numpy as np

PAD_EPS = float(np.float32(1e-8))


def trajectory_1(v0: float, a: float, t: int, n: int, dt: float) -> float:
    r = 0.0
    if n <= t:
        r = v0 + a * n * dt
    if n > t:
        r = v0 + a * t * dt
    return r


class VelocitySchedule:
    """Yields solve_v{x,y,z} for the steady state and each step, reproducing the pad."""

    def __init__(self, traj, dt):
        self.traj = [(float(t.v0), float(t.accel), int(t.n_accel)) for t in traj]
        self.dt = float(dt)
        self.acc = [0.0, 0.0, 0.0]
        self.v = [trajectory_1(v0, a, n, 0, self.dt) for (v0, a, n) in self.traj]

    def steady(self):
        return list(self.v)

    def step(self, counter: int):
        out = []
        for d, (v0, a, n) in enumerate(self.traj):
            if counter == 1:
                if a * self.dt < v0 * PAD_EPS:
                    self.acc[d] = self.v[d] * PAD_EPS / self.dt
            else:
                self.acc[d] = 0.0
            out.append(trajectory_1(v0, a + self.acc[d], n, counter, self.dt))
        self.v = out
        return list(out)


def excitation_scale(exc, t: float) -> float:
    if exc is None:
        return 1.0
    kind, f, ph = exc
    if kind == "cos":
        return math.cos(2.0 * math.pi * f * t + ph)
    return math.sin(2.0 * math.pi * f * t + ph)


def scaled_field(B, G, exc, t):
    """(B, G) in effect at time t; exact copies of the inputs when there is no excitation."""
    s = excitation_scale(exc, t)
    B = np.asarray(B, dtype=np.float64).reshape(3)
    G = np.asarray(G, dtype=np.float64).reshape(9)
    if s == 1.0:
        return B.copy(), G.copy()
    return B * s, G * s
