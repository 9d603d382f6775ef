"""Frame velocity and excitation schedule of a run (host-side scalars).

trajectory_1 (3D/QMS_3D.f90:2331-2350): v(n) = v0 + a*n*dt while n <= t,
v0 + a*t*dt afterwards.  The first transient step adds a small acceleration
"pad" when a*dt < v0*1E-8 (F:1428-1449); 1E-8 is a default-real (single
precision) literal and the pad state is static storage that starts at zero.
The same velocity drives the steady state (n = 0, F:431-433).

Trajectory types 2 (harmonic, v(n) = amp sin(2 pi f n dt + phase)) and 3 (a
per-step velocity table, the last entry held) extend the reference, which
stops on them (F:135-151).  The pad belongs to type 1: its test reads that
type's acceleration and initial velocity, so axes of the other types get none.

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


def trajectory_2(amp: float, f: float, phase: float, n: int, dt: float) -> float:
    """Harmonic frame motion: amp * sin(2 pi f t + phase) at t = n dt."""
    return amp * math.sin(2.0 * math.pi * f * (n * dt) + phase)


def trajectory_3(table, n: int) -> float:
    """Tabulated frame velocity: table[n], the last entry held after the table ends."""
    return float(table[min(n, len(table) - 1)])


class VelocitySchedule:
    """Yields solve_v{x,y,z} for the steady state and each step, reproducing the pad."""

    def __init__(self, traj, dt):
        self.traj = list(traj)
        self.dt = float(dt)
        self.acc = [0.0, 0.0, 0.0]
        self.v = [self._velocity(t, 0, 0.0) for t in self.traj]

    def _velocity(self, t, n, pad):
        kind = getattr(t, "kind", 1)
        if kind == 2:
            return trajectory_2(float(t.amp), float(t.freq), float(t.phase), n, self.dt)
        if kind == 3:
            return trajectory_3(t.table, n)
        return trajectory_1(float(t.v0), float(t.accel) + pad, int(t.n_accel), n, self.dt)

    def steady(self):
        return list(self.v)

    def step(self, counter: int):
        out = []
        for d, t in enumerate(self.traj):
            if getattr(t, "kind", 1) == 1:
                if counter == 1:
                    if float(t.accel) * self.dt < float(t.v0) * PAD_EPS:
                        self.acc[d] = self.v[d] * PAD_EPS / self.dt
                else:
                    self.acc[d] = 0.0
            out.append(self._velocity(t, counter, self.acc[d]))
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
