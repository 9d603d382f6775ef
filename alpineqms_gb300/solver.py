"""Python-side handle over libqms_gb300 (one solve = one grid resident on one GPU)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import (QMS_FIELD_CUBES, QMS_FIELD_SLICE, QMS_PREC_FP64, QMS_PREC_MIXED, QmsDesc, QmsProfile, QmsStats,
                   check, dvec)

AXES = {"x": 0, "y": 1, "z": 2}


def default_desc(xs, ys, zs, dx, dy, dz, dt, precision="mixed", **kw) -> QmsDesc:
    L = _lib.load()
    d = QmsDesc()
    L.qms_default_desc(ctypes.byref(d), xs, ys, zs, dx, dy, dz, dt)
    d.precision = QMS_PREC_FP64 if precision == "fp64" else QMS_PREC_MIXED
    for k, v in kw.items():
        if v is not None:
            setattr(d, k, v)
    return d


def device_bytes(desc: QmsDesc) -> int:
    return int(_lib.load().qms_device_bytes(ctypes.byref(desc)))


class QMSSolver:
    """Owns one qms_handle: materials, the resident solution x = [Ax|Ay|Az|V] and its workspace."""

    def __init__(self, desc: QmsDesc):
        self.L = _lib.load()
        self.desc = desc
        h = ctypes.c_void_p()
        rc = self.L.qms_create(ctypes.byref(desc), ctypes.byref(h))
        check(rc, None, "qms_create")
        self.h = h
        self.xs, self.ys, self.zs = desc.xs, desc.ys, desc.zs
        self.n = int(self.L.qms_n_dims(desc.xs, desc.ys, desc.zs))

    # ------------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.L.qms_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------
    def set_geometry_f64(self, geom: np.ndarray, table7: np.ndarray):
        geom = np.ascontiguousarray(geom, dtype=np.float64).reshape(-1)
        tab = np.ascontiguousarray(table7, dtype=np.float64).reshape(-1, 7)
        check(self.L.qms_set_geometry_f64(self.h, geom.ctypes.data, tab.ctypes.data, tab.shape[0]), self.h,
              "qms_set_geometry_f64")

    def set_materials(self, slots: np.ndarray, rows6: np.ndarray):
        slots = np.ascontiguousarray(slots, dtype=np.uint8).reshape(-1)
        rows = np.ascontiguousarray(rows6, dtype=np.float64).reshape(-1, 6)
        check(self.L.qms_set_materials(self.h, slots.ctypes.data, rows.ctypes.data, rows.shape[0]), self.h,
              "qms_set_materials")

    def steady(self, v, B, G):
        check(self.L.qms_steady(self.h, dvec(v), dvec(B), dvec(np.reshape(G, 9))), self.h, "qms_steady")
        return self.stats()

    def step(self, v, B, G):
        check(self.L.qms_step(self.h, dvec(v), dvec(B), dvec(np.reshape(G, 9))), self.h, "qms_step")
        return self.stats()

    def stats(self) -> dict:
        s = QmsStats()
        check(self.L.qms_get_stats(self.h, ctypes.byref(s)), self.h, "qms_get_stats")
        return dict(outer=s.outer_iterations, inner=s.inner_iterations, r0=s.initial_residual,
                    r=s.final_residual, status=s.status, step_graph=s.step_graph, start_ls=s.start_ls,
                    start_coef=list(s.start_coef), start_base=s.start_base, start_pred=s.start_pred)

    def fields(self):
        """(Hx, Hy, Hz) cubes, each (xs, ys, zs) Fortran-ordered views."""
        nc = self.xs * self.ys * self.zs
        out = np.empty(3 * nc, np.float64)
        check(self.L.qms_get_fields(self.h, QMS_FIELD_CUBES, 0, 1, out.ctypes.data), self.h, "qms_get_fields")
        return [out[q * nc:(q + 1) * nc].reshape((self.xs, self.ys, self.zs), order="F") for q in range(3)]

    def slices(self, axis: str, index: int):
        n1 = self.ys if axis == "x" else self.xs
        n2 = self.ys if axis == "z" else self.zs
        m = n1 * n2
        out = np.empty(3 * m, np.float64)
        check(self.L.qms_get_fields(self.h, QMS_FIELD_SLICE, AXES[axis], index, out.ctypes.data), self.h,
              "qms_get_fields")
        return [out[q * m:(q + 1) * m].reshape((n1, n2), order="F") for q in range(3)]

    def slice_shape(self, axis: str):
        n1 = self.ys if axis == "x" else self.xs
        n2 = self.ys if axis == "z" else self.zs
        return n1, n2

    def fields_async(self, which: int, axis: str, index: int, out: "PinnedBuffer", slot: int):
        """Start forming H (cubes, or the slice of `axis`/`index`) and copying it into `out`
        without waiting; the copy overlaps the handle's next calls.  fields_sync(slot) waits."""
        check(self.L.qms_get_fields_async(self.h, which, AXES.get(axis, 0), index, out.ptr, slot), self.h,
              "qms_get_fields_async")

    def fields_sync(self, slot: int):
        """Waits for the copy of `slot` (may be called from another thread)."""
        check(self.L.qms_fields_sync(self.h, slot), self.h, "qms_fields_sync")

    def get_state(self) -> np.ndarray:
        x = np.empty(self.n, np.float64)
        check(self.L.qms_get_state(self.h, x.ctypes.data), self.h, "qms_get_state")
        return x

    def get_rhs(self) -> np.ndarray:
        x = np.empty(self.n, np.float64)
        check(self.L.qms_get_rhs(self.h, x.ctypes.data), self.h, "qms_get_rhs")
        return x

    def set_state(self, x: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float64)
        assert x.size == self.n
        check(self.L.qms_set_state(self.h, x.ctypes.data), self.h, "qms_set_state")

    def residual_norm(self, transient: bool, v) -> float:
        out = ctypes.c_double()
        check(self.L.qms_residual_norm(self.h, 1 if transient else 0, dvec(v), ctypes.byref(out)), self.h,
              "qms_residual_norm")
        return out.value

    # instrumentation
    def profile_enable(self, on=True):
        check(self.L.qms_profile_enable(self.h, 1 if on else 0), self.h, "qms_profile_enable")

    def profile(self) -> dict:
        p = QmsProfile()
        check(self.L.qms_get_profile(self.h, ctypes.byref(p)), self.h, "qms_get_profile")
        return {k: getattr(p, k) for k, _ in QmsProfile._fields_}

    def stream_ptr(self) -> int:
        return int(self.L.qms_get_stream(self.h) or 0)

    # device-pointer verification entry points (torch tensors or raw addresses)
    def assemble_csr(self, transient, v, B, G, d_xprev, d_ia, d_ja, d_a, d_b):
        check(self.L.qms_assemble_csr(self.h, 1 if transient else 0, dvec(v), dvec(B), dvec(np.reshape(G, 9)),
                                      d_xprev or None, d_ia, d_ja, d_a, d_b), self.h, "qms_assemble_csr")

    def apply(self, transient, v, fp32, d_x, d_y):
        check(self.L.qms_apply(self.h, 1 if transient else 0, dvec(v), 1 if fp32 else 0, d_x, d_y), self.h,
              "qms_apply")

    def csr_spmv(self, d_ia, d_ja, d_a, d_x, d_y):
        check(self.L.qms_csr_spmv(self.h, d_ia, d_ja, d_a, d_x, d_y), self.h, "qms_csr_spmv")


class PinnedBuffer:
    """Page-locked host memory (qms_pinned_alloc) seen as a float64 numpy array."""

    def __init__(self, n: int):
        self.L = _lib.load()
        self.n = int(n)
        self.ptr = self.L.qms_pinned_alloc(self.n * 8)
        if not self.ptr:
            raise MemoryError(f"qms_pinned_alloc({self.n * 8}) failed")
        self.array = np.ctypeslib.as_array(ctypes.cast(self.ptr, ctypes.POINTER(ctypes.c_double)), shape=(self.n,))

    def close(self):
        if getattr(self, "ptr", None):
            self.array = None
            self.L.qms_pinned_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
