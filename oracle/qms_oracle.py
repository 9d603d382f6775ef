"""CPU oracle for the QMS_3D per-step hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline / reference legs import this module; the product
package ``alpineqms_gb300`` never does.

What it is:

* a ctypes wrapper over ``qms_oracle.c``, a C restatement of the reference's
  material averaging (3D/QMS_3D.f90:234-269), CSR assembly (F:448-1312 steady,
  F:1457-2191 transient), H computation (F:1320-1376) and trajectory
  (F:2331-2350);
* ``DirectSolver``: SciPy SuperLU standing in for MKL PARDISO (mtype 11,
  F:1314-1317, F:2193-2203).  PARDISO is closed source and absent here; the
  reference factors once per matrix (phase 13 / 23) and back-substitutes when
  only the RHS changed (phase 33).  ``simulate`` mirrors that reuse;
* ``simulate``: the reference's main program flow (steady init, then
  ``Nt`` backward-Euler steps, H dumps with the same cadence, F:1378-1404,
  F:2274-2300).

The C restatement is pinned against golden vectors that were produced by
executing the reference's own Fortran source (tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "qms_oracle.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libqms_oracle.so")

MU0 = 1.25663706e-6  # F:22

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile qms_oracle.c with gcc (-ffp-contract=off keeps source-order rounding)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", tmp, SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            i64p = ctypes.POINTER(ctypes.c_int64)
            dp = ctypes.c_void_p
            L.qmso_sizes.argtypes = [ctypes.c_int] * 3 + [i64p, i64p, i64p]
            L.qmso_sizes.restype = None
            L.qmso_materials.argtypes = [ctypes.c_int] * 3 + [dp, ctypes.c_int, dp] + [dp] * 6
            L.qmso_materials.restype = ctypes.c_int
            L.qmso_assemble.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_double] * 3 + [dp] * 6
                                        + [ctypes.c_int, ctypes.c_double, dp, dp, dp, dp, dp, dp, dp, dp])
            L.qmso_assemble.restype = ctypes.c_int64
            L.qmso_hfield.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 3 + [dp] * 7
            L.qmso_hfield.restype = None
            L.qmso_trajectory.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double]
            L.qmso_trajectory.restype = ctypes.c_double
            L.qmso_step_velocity.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_double,
                                             ctypes.POINTER(ctypes.c_double)]
            L.qmso_step_velocity.restype = ctypes.c_double
            L.qmso_num_threads.argtypes = []
            L.qmso_num_threads.restype = ctypes.c_int
            _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


def num_threads() -> int:
    return lib().qmso_num_threads()


# --------------------------------------------------------------------------
def sizes(xs, ys, zs):
    """(n_dims, nnz, exact_nn) of F:172-181 and the row predicates."""
    n, nnz, ex = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    lib().qmso_sizes(xs, ys, zs, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(ex))
    return n.value, nnz.value, ex.value


def block_offsets(xs, ys, zs):
    """0-based start rows of the Ax, Ay, Az, V blocks and n_dims."""
    Nx, Ny, Nz = xs + 1, ys + 1, zs + 1
    Nn = Nx * Ny * Nz
    oY = Nn - Ny * Nz
    oZ = 2 * Nn - Ny * Nz - Nx * Nz
    oV = 3 * Nn - Ny * Nz - Nx * Nz - Nx * Ny
    n = 4 * Nn - Ny * Nz - Nx * Nz - Nx * Ny
    return 0, oY, oZ, oV, n


def materials(xs, ys, zs, geom, props):
    """geom: float64 IDs, xs*ys*zs in F-order; props: (nmat, 7) id, mur xyz, sigma xyz.
    Returns dict of node-sized F-order float64 arrays mu_x..sig_z (F:193-269)."""
    geom = np.ascontiguousarray(np.asarray(geom, dtype=np.float64).reshape(-1, order="F") if np.ndim(geom) == 3
                                else np.asarray(geom, dtype=np.float64))
    props = np.ascontiguousarray(np.asarray(props, dtype=np.float64).reshape(-1, 7))
    Nn = (xs + 1) * (ys + 1) * (zs + 1)
    out = {k: np.empty(Nn, np.float64) for k in ("mu_x", "mu_y", "mu_z", "sig_x", "sig_y", "sig_z")}
    rc = lib().qmso_materials(xs, ys, zs, _p(geom), props.shape[0], _p(props),
                              *[_p(out[k]) for k in ("mu_x", "mu_y", "mu_z", "sig_x", "sig_y", "sig_z")])
    if rc != 0:
        raise ValueError("geometry holds a material ID that is negative or above the largest table ID")
    return out


def assemble(xs, ys, zs, dx, dy, dz, coefs, transient, dt, v, B, G, x_prev=None):
    """CSR (1-based int32 ia/ja, float64 a) and RHS b of F:448-1296 / F:1457-2191."""
    n, nnz, _ = sizes(xs, ys, zs)
    ia = np.empty(n + 1, np.int32)
    ja = np.empty(nnz, np.int32)
    a = np.empty(nnz, np.float64)
    b = np.empty(n, np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    G = np.ascontiguousarray(np.asarray(G, dtype=np.float64).reshape(9))
    xp = np.zeros(n, np.float64) if x_prev is None else np.ascontiguousarray(x_prev, dtype=np.float64)
    got = lib().qmso_assemble(xs, ys, zs, dx, dy, dz,
                              *[_p(coefs[k]) for k in ("mu_x", "mu_y", "mu_z", "sig_x", "sig_y", "sig_z")],
                              1 if transient else 0, dt, _p(v), _p(B), _p(G), _p(xp),
                              _p(ia), _p(ja), _p(a), _p(b))
    if got == -1:
        raise OverflowError("nnz exceeds the int32 CSR of the reference")
    if got == -2:
        raise RuntimeError("CSR self-check failed (unsorted row or negative column)")
    assert got == nnz
    return ia, ja, a, b


def hfield(xs, ys, zs, dx, dy, dz, coefs, x):
    """Hx, Hy, Hz at cell centres (F:1346-1376), each xs*ys*zs F-order flat."""
    nc = xs * ys * zs
    H = [np.empty(nc, np.float64) for _ in range(3)]
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().qmso_hfield(xs, ys, zs, dx, dy, dz, _p(coefs["mu_x"]), _p(coefs["mu_y"]), _p(coefs["mu_z"]),
                      _p(x), *[_p(h) for h in H])
    return H


def trajectory(v, a, t, n, dt):
    return lib().qmso_trajectory(v, a, t, n, dt)


def step_velocity(v0, a, t, counter, dt, prev_v, acc_state):
    """Returns (velocity, new acc_state) for transient step `counter` (F:1428-1449)."""
    st = ctypes.c_double(acc_state)
    v = lib().qmso_step_velocity(v0, a, t, counter, dt, prev_v, ctypes.byref(st))
    return v, st.value


def excitation_scale(exc, t):
    """Background-field scale s(t).  exc None => 1 (the reference's static B_in)."""
    if exc is None:
        return 1.0
    kind, f, ph = exc
    if kind == "cos":
        return math.cos(2.0 * math.pi * f * t + ph)
    if kind == "sin":
        return math.sin(2.0 * math.pi * f * t + ph)
    raise ValueError(kind)


def to_scipy(ia, ja, a, n):
    import scipy.sparse as sp
    return sp.csr_matrix((a, ja.astype(np.int64) - 1, ia.astype(np.int64) - 1), shape=(n, n))


class DirectSolver:
    """SuperLU in place of PARDISO: factor on demand, reuse while the matrix is unchanged.

    The rows of this system span ~20 decades (air V rows carry the 1e-12 S/m
    conductivity floor, F:1237-1281; A rows ~1e12), and plain LU on it leaves
    scaled residuals near 1e-9 with errors up to 1e-5 in A.  The oracle therefore
    factors the row-equilibrated matrix D^-1 M (D = |diag M|) and refines the
    solution with FP64 residuals until the scaled residual stops improving
    (~1e-16).  The electric potential of an isolated conductor is still fixed
    only through the 1e-12 S/m floor (a mode ~19 decades below the conductor
    scale), so V carries an arbitrary constant per isolated conductor in any
    FP64 solve; that constant changes neither A nor H (sigma*grad V vanishes
    on it), and comparisons of V use the edge current sigma*grad V.
    """

    def __init__(self):
        self.lu = None

    def factor(self, ia, ja, a, n, symmetric_mode=True):
        import scipy.sparse as sp
        import scipy.sparse.linalg as spl
        A = to_scipy(ia, ja, a, n)
        self.A = A
        self.d = np.abs(A.diagonal())
        As = (sp.diags(1.0 / self.d) @ A).tocsc()
        if symmetric_mode:
            # diagonal pivots on the equilibrated matrix with a symmetric (A+A^T) ordering:
            # far less fill than column ordering with partial pivoting on this system
            self.lu = spl.splu(As, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0,
                               options={"SymmetricMode": True})
        else:
            self.lu = spl.splu(As, permc_spec="COLAMD")
        self._As = As

    def solve(self, b, max_refine=8):
        b = np.asarray(b, dtype=np.float64)
        x = self._refine(b, max_refine)
        if not self._ok(b, x):              # pivoting trouble: fall back to partial pivoting
            import scipy.sparse.linalg as spl
            self.lu = spl.splu(self._As, permc_spec="COLAMD")
            x = self._refine(b, max_refine)
        return x

    def _ok(self, b, x):
        r = (b - self.A @ x) / self.d
        return np.isfinite(r).all() and np.linalg.norm(r) <= 1e-13 * max(np.linalg.norm(x), 1e-300)

    def _refine(self, b, max_refine):
        x = self.lu.solve(b / self.d)
        best = None
        for _ in range(max_refine):
            r = (b - self.A @ x) / self.d
            nr = np.linalg.norm(r)
            if not np.isfinite(nr) or (best is not None and nr >= 0.5 * best):
                break
            best = nr if best is None else min(best, nr)
            x = x + self.lu.solve(r)
        return x


def edge_current_from_v(xs, ys, zs, dx, dy, dz, coefs, x):
    """sigma_edge * dV/dh on every x-, y- and z-edge: the way V enters the A rows
    (F:595-607, F:769-781, F:943-955).  Used to compare V up to the floating
    constant of isolated conductors."""
    Nx, Ny, Nz = xs + 1, ys + 1, zs + 1
    _, _, _, oV, _ = block_offsets(xs, ys, zs)
    V = np.asarray(x[oV:], np.float64).reshape((Nx, Ny, Nz), order="F")
    sx = coefs["sig_x"].reshape((Nx, Ny, Nz), order="F")
    sy = coefs["sig_y"].reshape((Nx, Ny, Nz), order="F")
    sz = coefs["sig_z"].reshape((Nx, Ny, Nz), order="F")
    jx = sx[:xs] * (V[1:] - V[:-1]) / dx
    jy = sy[:, :ys] * (V[:, 1:] - V[:, :-1]) / dy
    jz = sz[:, :, :zs] * (V[:, :, 1:] - V[:, :, :-1]) / dz
    return np.concatenate([jx.ravel(order="F"), jy.ravel(order="F"), jz.ravel(order="F")])


def simulate(p, geom, steps=None, on_step=None, keep_states=False):
    """Run the reference algorithm on CPU with a direct solver.

    p: dict with xs, ys, zs, dx, dy, dz, dt, Nt, B (3), G (3x3), traj (3 x (v0, a, nacc)),
       props (nmat, 7), optional excitation (kind, f, phase).  An optional ``velocities``
       array ((steps + 1) x 3: the steady state's, then each step's) replaces the type-1
       trajectory: the frame motions the reference stops on (F:135-151) enter its
       assembly the same way, as one velocity per axis and step (F:431-433, F:1447-1449).
    Yields nothing; calls on_step(counter, x, H) for the steady state (counter 0)
    and each transient step.  Returns the list of (counter, x, H) if keep_states.
    """
    xs, ys, zs = p["xs"], p["ys"], p["zs"]
    dx, dy, dz, dt = p["dx"], p["dy"], p["dz"], p["dt"]
    nt = p["Nt"] if steps is None else steps
    coefs = materials(xs, ys, zs, geom, p["props"])
    traj = p["traj"]
    B0 = np.asarray(p["B"], np.float64)
    G0 = np.asarray(p["G"], np.float64).reshape(9)
    exc = p.get("excitation")
    n, _, _ = sizes(xs, ys, zs)
    out = []

    def scaled(t):
        s = excitation_scale(exc, t)
        if s == 1.0:
            return B0, G0
        return B0 * s, G0 * s

    vel = p.get("velocities")
    if vel is not None:
        vel = np.asarray(vel, np.float64).reshape(-1, 3)
        v = vel[0].copy()
    else:
        v = np.array([trajectory(traj[d][0], traj[d][1], int(traj[d][2]), 0, dt) for d in range(3)])
    Bs, Gs = scaled(0.0)
    ia, ja, a, b = assemble(xs, ys, zs, dx, dy, dz, coefs, False, dt, v, Bs, Gs)
    ds = DirectSolver()
    ds.factor(ia, ja, a, n)
    x = ds.solve(b)
    H = hfield(xs, ys, zs, dx, dy, dz, coefs, x)
    if on_step:
        on_step(0, x, H)
    if keep_states:
        out.append((0, x.copy(), [h.copy() for h in H]))
    ov = v.copy()
    acc = [0.0, 0.0, 0.0]
    dt_solver = DirectSolver()
    for counter in range(1, nt + 1):
        nv = np.empty(3)
        for d in range(3):
            if vel is not None:
                nv[d] = vel[counter, d]
            else:
                nv[d], acc[d] = step_velocity(traj[d][0], traj[d][1], int(traj[d][2]), counter, dt, v[d], acc[d])
        v = nv
        Bs, Gs = scaled(counter * dt)
        ia, ja, a, b = assemble(xs, ys, zs, dx, dy, dz, coefs, True, dt, v, Bs, Gs, x)
        if not (np.all(ov == v) and counter > 1):       # F:2193-2203 phase 23 vs 33
            dt_solver.factor(ia, ja, a, n)
        x = dt_solver.solve(b)
        ov = v.copy()
        H = hfield(xs, ys, zs, dx, dy, dz, coefs, x)
        if on_step:
            on_step(counter, x, H)
        if keep_states:
            out.append((counter, x.copy(), [h.copy() for h in H]))
    return out
