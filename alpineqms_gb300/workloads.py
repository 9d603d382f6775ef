"""Seeded synthetic workloads, expressed in the reference's inputs grammar.

Every generator returns ``(QMSInputs, geom)`` where ``geom`` is the float64
material-ID cube flattened in Fortran order (what geom.bin holds,
3D/master.py:68-77).  ``inputs_text`` writes the matching ``inputs.txt`` in
the positional format of master.py:23-66 (+ the optional trailing excitation
line).  Random choices use ``numpy.random.Generator(PCG64(seed))``.

Workloads (grid / materials / excitation / steps):
  plain_block_32     32^3, 1 mm, centred 12x12x8 copper block (sigma 5.8e7),
                     B0 z 1 mT at 1 kHz (cos), v = 0, steady + 20 @ 1e-5 s
  inclusions_96      96^3, 0.5 mm, 24 random ellipsoids (semi-axes U[3,15]
                     cells, mu_r logU[1,1e3], sigma logU[1e5,6e7]), B0 x 5 mT
                     500 Hz, 100 @ 2e-5 s
  moving_plate_256   256^3, 1 mm, aluminium plate 200x200x10 (sigma 3.5e7)
                     in a static field Bz = 10 mT + 0.1 T/m z-gradient
                     (gxx = gyy = -0.05 T/m keep it divergence free); the
                     frame velocity ramps from 0 to -10 m/s x in the first step
                     (trajectory type 1: v0 = 0, a = -1e6 m/s^2, n_acc = 1),
                     i.e. the plate starts moving at +10 m/s at t = 0;
                     steady (v = 0) + 200 @ 1e-5 s
  serving request    {48^3, 64^3, 96^3, 128^3, 128x64x32}, 8-32 ellipsoids
                     as inclusions_96, B0 in a random direction, 1-10 mT,
                     f log-uniform in [50, 5000] Hz, 50 @ 1/(40 f)
  laminated_core     512x512x256, 0.25 mm, 40 steel laminations (mu_r 2000,
                     sigma 2e6, 5 cells) with 1-cell gaps, B0 x 0.5 T 60 Hz,
                     steady + 100 @ 1.6e-4 s
"""
from __future__ import annotations

import numpy as np

from .inputs import Material, QMSInputs, Trajectory

STATIC = None


def _inputs(size, h, dt, nt, B, G, traj, mats, excitation, slice_axis="z", slice_index=None, save_all="no", tt=1):
    xs, ys, zs = size
    if slice_index is None:
        slice_index = {"x": xs, "y": ys, "z": zs}[slice_axis] // 2
    return QMSInputs(xs, ys, zs, h, h, h, dt, nt, tt, slice_axis, slice_index, save_all, tuple(B),
                     tuple(tuple(r) for r in np.reshape(G, (3, 3))), tuple(Trajectory(1, *t) for t in traj),
                     [Material(float(m[0]), tuple(m[1]), tuple(m[2])) for m in mats], "geom.bin", excitation)


def plain_block_32(nt=20):
    xs = ys = zs = 32
    geom = np.zeros((xs, ys, zs))
    geom[10:22, 10:22, 12:20] = 1
    inp = _inputs((xs, ys, zs), 1e-3, 1e-5, nt, (0.0, 0.0, 1e-3), np.zeros(9), [(0.0, 0.0, 0)] * 3,
                  [(1, (1.0, 1.0, 1.0), (5.8e7, 5.8e7, 5.8e7))], ("cos", 1000.0, 0.0))
    return inp, geom.flatten(order="F")


def paint_ellipsoids(shape, n, rng, semi=(3, 15)):
    """n ellipsoids with centres uniform in the non-Dirichlet interior (3..N-2),
    semi-axes uniform in `semi` cells, painted in order (later ones overwrite)."""
    xs, ys, zs = shape
    geom = np.zeros(shape)
    I, J, K = np.meshgrid(np.arange(xs) + 0.5, np.arange(ys) + 0.5, np.arange(zs) + 0.5, indexing="ij")
    for m in range(1, n + 1):
        c = [rng.uniform(3, s - 2) for s in shape]
        a = rng.uniform(semi[0], semi[1], 3)
        inside = ((I - c[0]) / a[0]) ** 2 + ((J - c[1]) / a[1]) ** 2 + ((K - c[2]) / a[2]) ** 2 <= 1.0
        geom[inside] = m
    # keep the two-layer Dirichlet shell in air
    geom[:2, :, :] = 0; geom[-2:, :, :] = 0
    geom[:, :2, :] = 0; geom[:, -2:, :] = 0
    geom[:, :, :2] = 0; geom[:, :, -2:] = 0
    return geom


def random_materials(n, rng):
    mats = []
    for m in range(1, n + 1):
        mu = float(10 ** rng.uniform(0.0, 3.0))
        sg = float(10 ** rng.uniform(5.0, np.log10(6e7)))
        mats.append((m, (mu, mu, mu), (sg, sg, sg)))
    return mats


def inclusions_96(seed=2, nt=100, size=96):
    rng = np.random.default_rng(np.random.PCG64(seed))
    shape = (size, size, size)
    geom = paint_ellipsoids(shape, 24, rng)
    mats = random_materials(24, rng)
    inp = _inputs(shape, 0.5e-3, 2e-5, nt, (5e-3, 0.0, 0.0), np.zeros(9), [(0.0, 0.0, 0)] * 3, mats,
                  ("cos", 500.0, 0.0))
    return inp, geom.flatten(order="F")


def moving_plate(size=256, nt=200, plate=(200, 200, 10), h=1e-3):
    xs = ys = zs = size
    geom = np.zeros((xs, ys, zs))
    px, py, pz = (min(plate[0], xs - 8), min(plate[1], ys - 8), min(plate[2], max(zs // 8, 1)))
    x0, y0, z0 = (xs - px) // 2, (ys - py) // 2, (zs - pz) // 2
    geom[x0:x0 + px, y0:y0 + py, z0:z0 + pz] = 1
    G = [-0.05, 0.0, 0.0, 0.0, -0.05, 0.0, 0.0, 0.0, 0.1]
    inp = _inputs((xs, ys, zs), h, 1e-5, nt, (0.0, 0.0, 1e-2), G, [(0.0, -1e6, 1), (0.0, 0.0, 0), (0.0, 0.0, 0)],
                  [(1, (1.0, 1.0, 1.0), (3.5e7, 3.5e7, 3.5e7))], STATIC)
    return inp, geom.flatten(order="F")


def moving_plate_256(nt=200):
    return moving_plate(256, nt)


SERVING_SIZES = ((48, 48, 48), (64, 64, 64), (96, 96, 96), (128, 128, 128), (128, 64, 32))


def serving_request(rng, sizes=SERVING_SIZES, nt=50, h=1e-3):
    shape = sizes[rng.integers(0, len(sizes))]
    nell = int(rng.integers(8, 33))
    geom = paint_ellipsoids(shape, nell, rng, semi=(3, max(4, min(15, min(shape) // 4))))
    mats = random_materials(nell, rng)
    d = rng.standard_normal(3)
    d /= np.linalg.norm(d)
    amp = rng.uniform(1e-3, 1e-2)
    f = float(10 ** rng.uniform(np.log10(50.0), np.log10(5000.0)))
    inp = _inputs(shape, h, 1.0 / (40.0 * f), nt, tuple(amp * d), np.zeros(9), [(0.0, 0.0, 0)] * 3, mats,
                  ("cos", f, 0.0))
    return inp, geom.flatten(order="F")


def laminated_core(nt=100, shape=(512, 512, 256), h=0.25e-3, laminations=40):
    xs, ys, zs = shape
    geom = np.zeros(shape)
    stack = laminations * 5 + laminations - 1
    z0 = (zs - stack) // 2
    mx, my = xs // 8, ys // 8
    for L in range(laminations):
        z = z0 + L * 6
        geom[mx:xs - mx, my:ys - my, z:z + 5] = 1
    inp = _inputs(shape, h, 1.6e-4, nt, (0.5, 0.0, 0.0), np.zeros(9), [(0.0, 0.0, 0)] * 3,
                  [(1, (2000.0, 2000.0, 2000.0), (2e6, 2e6, 2e6))], ("cos", 60.0, 0.0))
    return inp, geom.flatten(order="F")


WORKLOADS = {
    "plain_block_32": plain_block_32,
    "inclusions_96": inclusions_96,
    "moving_plate_256": moving_plate_256,
    "laminated_core": laminated_core,
}


def inputs_text(inp: QMSInputs) -> str:
    """inputs.txt in the positional grammar of 3D/master.py:23-66."""
    def r3(v):     # plain Python floats: numpy scalars would print as np.float64(...)
        return "{!r},{!r},{!r}".format(*(float(a) for a in v))
    L = [f"{inp.xs},{inp.ys},{inp.zs}", r3((inp.dx, inp.dy, inp.dz)), repr(float(inp.dt)), str(inp.nt),
         str(inp.tt), f"{inp.slice_axis},{inp.slice_index}", inp.save_all, r3(inp.B)]
    for row in inp.G:
        L.append(r3(row))
    for t in inp.traj:
        L.append(str(t.kind))
        if t.kind == 2:
            L.append(r3((t.amp, t.freq, t.phase)))
        elif t.kind == 3:
            L.append(str(len(t.table)))
            L.append(",".join(repr(float(v)) for v in t.table))
        else:
            L.append(f"{float(t.v0)!r},{float(t.accel)!r},{int(t.n_accel)}")
    L.append(str(len(inp.materials)))
    for m in inp.materials:
        L.append(repr(float(m.mat_id)))
        L.append(r3(m.mu_r))
        L.append(r3(m.sigma))
    L.append(inp.geom_name)
    if inp.excitation is not None:
        k, f, ph = inp.excitation
        L.append(f"excitation,{k},{float(f)!r},{float(ph)!r}")
    return "\n".join(L) + "\n"


def write_case(directory: str, inp: QMSInputs, geom: np.ndarray):
    import os
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, "inputs.txt"), "w") as f:
        f.write(inputs_text(inp))
    np.asarray(geom, dtype="<f8").tofile(os.path.join(directory, inp.geom_name))
