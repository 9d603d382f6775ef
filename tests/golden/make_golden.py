"""Generate golden fixtures by executing the reference program itself.

Run in a container where the reference checkout is mounted (the path is the
first argument, required).  For each case below this script:

1. writes ``inputs.txt`` and ``geom.bin`` in a scratch directory, in the
   grammar of 3D/master.py:16-77;
2. executes 3D/QMS_3D.f90 with ``fortran_exec`` (a Fortran-subset
   interpreter; no compiler exists here), routing every ``pardiso`` call to
   the oracle's direct solver (row-equilibrated SuperLU with FP64 refinement,
   standing in for MKL PARDISO) and recording the CSR arrays and right-hand
   side the program hands it;
3. saves, per case, ``<case>.npz`` holding: the inputs text and geometry, the
   1-based int32 ``ia``/``ja`` (checked identical for every solver call), and
   for each call its ``phase``, ``a`` values, ``b`` and solution ``x``; plus the
   bytes of every field dump the program wrote (Hx.bin ... Hz_all.bin).

The fixtures are small (grids of 6-9 cells per side).  They pin the CPU
oracle (oracle/qms_oracle.c) and the host-side dump writer; the GPU tests
then compare against the oracle.

Usage:  python tests/golden/make_golden.py /path/to/reference
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))

import fortran_exec  # noqa: E402

DUMPS = ("Hx.bin", "Hy.bin", "Hz.bin", "Hx_all.bin", "Hy_all.bin", "Hz_all.bin")


def inputs_text(c):
    L = []
    L.append("{},{},{}".format(*c["size"]))
    L.append("{!r},{!r},{!r}".format(*c["d"]))
    L.append(repr(c["dt"]))
    L.append(str(c["Nt"]))
    L.append(str(c["tt"]))
    L.append("{},{}".format(*c["slice"]))
    L.append(c["save_all"])
    L.append("{!r},{!r},{!r}".format(*c["B"]))
    for row in c["G"]:
        L.append("{!r},{!r},{!r}".format(*row))
    for (v0, a, n) in c["traj"]:
        L.append("1")
        L.append(f"{v0!r},{a!r},{n}")
    L.append(str(len(c["mats"])))
    for (mid, mur, sig) in c["mats"]:
        L.append(str(mid))
        L.append("{!r},{!r},{!r}".format(*mur))
        L.append("{!r},{!r},{!r}".format(*sig))
    L.append("geom.bin")
    return "\n".join(L) + "\n"


def cases():
    rng = np.random.default_rng(20261203)
    out = []
    # 1: anisotropic grid and spacing, accelerating frame (phase 23 every step),
    #    traceless symmetric gradient, y-slice, full dumps, tt = 2
    xs, ys, zs = 7, 8, 9
    geom = np.zeros((xs, ys, zs))
    geom[2:5, 2:6, 3:7] = 5
    geom[3:5, 4:6, 4:6] = 6
    geom[1, 1, 1] = 9          # an ID that is not in the table -> vacuum (F:243-244)
    out.append(dict(name="aniso_accel", size=(xs, ys, zs), d=(1.0e-3, 1.5e-3, 0.8e-3), dt=2.0e-5,
                    Nt=3, tt=2, slice=("y", 4), save_all="yes", B=(2.0e-3, -1.0e-3, 5.0e-3),
                    G=((0.05, 0.02, -0.01), (0.02, -0.03, 0.04), (-0.01, 0.04, -0.02)),
                    traj=((1.5, 200.0, 2), (-0.5, 0.0, 0), (0.25, -50.0, 5)),
                    mats=((5, (1.0, 2.0, 3.0), (5.8e7, 3.0e7, 1.0e7)),
                          (6, (50.0, 40.0, 30.0), (0.0, 1.0e5, 2.0e6)),
                          (9000, (1.0, 1.0, 1.0), (1.0, 1.0, 1.0))),
                    geom=geom))
    # 2: static frame (v = 0), conductor block, x-slice, no full dumps, constant
    #    v after step 1 (phase 33 path), tt = 1
    xs, ys, zs = 8, 8, 8
    geom = np.zeros((xs, ys, zs))
    geom[2:6, 2:6, 3:5] = 1
    out.append(dict(name="static_block", size=(xs, ys, zs), d=(1.0e-3, 1.0e-3, 1.0e-3), dt=1.0e-5,
                    Nt=3, tt=1, slice=("x", 4), save_all="no", B=(0.0, 0.0, 1.0e-3),
                    G=((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)),
                    traj=((0.0, 0.0, 0), (0.0, 0.0, 0), (0.0, 0.0, 0)),
                    mats=((1, (1.0, 1.0, 1.0), (5.8e7, 5.8e7, 5.8e7)),),
                    geom=geom))
    # 3: random materials (every cell), moving frame with a 1-step ramp, z-slice
    xs, ys, zs = 6, 7, 6
    geom = rng.integers(0, 4, size=(xs, ys, zs)).astype(np.float64)
    mats = []
    for mid in (1, 2, 3):
        mats.append((mid, tuple(float(10 ** rng.uniform(0, 3)) for _ in range(3)),
                     tuple(float(10 ** rng.uniform(5, 7.7)) for _ in range(3))))
    out.append(dict(name="random_ramp", size=(xs, ys, zs), d=(2.0e-3, 2.0e-3, 2.0e-3), dt=5.0e-5,
                    Nt=2, tt=1, slice=("z", 3), save_all="yes", B=(1.0e-2, 0.0, 0.0),
                    G=((0.0, 0.0, 0.1), (0.0, -0.05, 0.0), (0.1, 0.0, 0.05)),
                    traj=((0.0, -2.0e5, 1), (0.0, 0.0, 0), (0.0, 0.0, 0)),
                    mats=tuple(mats), geom=geom))
    return out


def run_case(src, c, workdir):
    import qms_oracle

    os.makedirs(workdir, exist_ok=True)
    txt = inputs_text(c)
    with open(os.path.join(workdir, "inputs.txt"), "w") as f:
        f.write(txt)
    c["geom"].astype("<f8").flatten(order="F").tofile(os.path.join(workdir, "geom.bin"))
    calls = []
    state = {"lu": None}

    def hook(phase, n, a, ia, ja, b, x):
        n = int(n)
        if int(phase) == -1:
            return
        nnz = int(ia[n]) - 1
        if int(phase) in (13, 23):
            state["lu"] = qms_oracle.DirectSolver()
            state["lu"].factor(ia[:n + 1].astype(np.int32), ja[:nnz].astype(np.int32), a[:nnz].copy(), n)
        sol = state["lu"].solve(b.copy())
        x[:] = sol
        calls.append(dict(phase=int(phase), ia=ia[:n + 1].astype(np.int32).copy(),
                          ja=ja[:nnz].astype(np.int32).copy(), a=a[:nnz].copy(), b=b.copy(), x=sol.copy()))

    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        io = fortran_exec.run_program(src, workdir, ["QMS_3D", "inputs.txt"], hook)
    dumps = {}
    for nm in DUMPS:
        pth = os.path.join(workdir, nm)
        if os.path.exists(pth):
            dumps[nm] = np.frombuffer(open(pth, "rb").read(), dtype=np.uint8)
    return txt, calls, dumps, io.stdout


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/reference  (the AlpineQMS checkout)")
    ref = sys.argv[1]
    src = os.path.join(ref, "3D", "QMS_3D.f90")
    for c in cases():
        with tempfile.TemporaryDirectory() as td:
            txt, calls, dumps, stdout = run_case(src, c, td)
        ia0, ja0 = calls[0]["ia"], calls[0]["ja"]
        for cl in calls[1:]:
            assert np.array_equal(cl["ia"], ia0) and np.array_equal(cl["ja"], ja0)
        payload = dict(inputs_txt=np.frombuffer(txt.encode(), dtype=np.uint8),
                       geom=c["geom"].astype(np.float64), ia=ia0, ja=ja0,
                       phases=np.array([cl["phase"] for cl in calls], np.int32))
        for q, cl in enumerate(calls):
            payload[f"a{q}"] = cl["a"]
            payload[f"b{q}"] = cl["b"]
            payload[f"x{q}"] = cl["x"]
        for nm, data in dumps.items():
            payload["dump_" + nm.replace(".", "_")] = data
        out = os.path.join(HERE, c["name"] + ".npz")
        np.savez_compressed(out, **payload)
        print(f"{c['name']}: n={len(ia0) - 1} nnz={len(ja0)} calls={[cl['phase'] for cl in calls]} "
              f"dumps={sorted(dumps)} -> {os.path.relpath(out)} ({os.path.getsize(out)} B)")


if __name__ == "__main__":
    main()
