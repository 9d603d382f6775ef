"""ctypes binding of libqms_gb300.so (declarations in include/qms.h).

The library must have been built (``python -m alpineqms_gb300.build`` or
``__graft_entry__.build()``); there is no fallback implementation, so a
missing library raises ``QMSLibraryError`` instead of computing anything on
the CPU.
"""
from __future__ import annotations

import ctypes
import os
import threading

from .build import LIB

_lock = threading.Lock()
_lib = None


class QMSLibraryError(RuntimeError):
    pass


class QmsDesc(ctypes.Structure):
    _fields_ = [("xs", ctypes.c_int), ("ys", ctypes.c_int), ("zs", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("dt", ctypes.c_double),
                ("precision", ctypes.c_int),
                ("tol", ctypes.c_double),
                ("max_outer", ctypes.c_int),
                ("max_inner", ctypes.c_int),
                ("inner_rtol", ctypes.c_double),
                ("check_every", ctypes.c_int),
                ("device", ctypes.c_int),
                ("precond", ctypes.c_int),
                ("mg_sweeps", ctypes.c_int),
                ("mg_omega", ctypes.c_double),
                ("mg_vshift", ctypes.c_double),
                ("krylov", ctypes.c_int),
                ("gmres_m", ctypes.c_int),
                ("use_graphs", ctypes.c_int), ("mg_region_cut", ctypes.c_double),
                ("mg_alpha", ctypes.c_double), ("mg_coupling", ctypes.c_int),
                ("mg_coarse_sweeps", ctypes.c_int), ("mg_v_sweeps", ctypes.c_int),
                ("mg_tail_points", ctypes.c_int), ("extrapolate", ctypes.c_int),
                ("mg_v_coarse_cut", ctypes.c_double), ("gm_first_extend", ctypes.c_int),
                ("tol_v", ctypes.c_double), ("start_ls", ctypes.c_int)]


class QmsStats(ctypes.Structure):
    _fields_ = [("outer_iterations", ctypes.c_int),
                ("inner_iterations", ctypes.c_int),
                ("initial_residual", ctypes.c_double),
                ("final_residual", ctypes.c_double),
                ("status", ctypes.c_uint), ("step_graph", ctypes.c_int),
                ("start_ls", ctypes.c_int), ("start_coef", ctypes.c_double * 4),
                ("start_base", ctypes.c_double), ("start_pred", ctypes.c_double)]


class QmsProfile(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_int64),
                ("op32_launches", ctypes.c_int64), ("op32_ms", ctypes.c_double), ("op32_bytes", ctypes.c_double),
                ("op64_launches", ctypes.c_int64), ("op64_ms", ctypes.c_double), ("op64_bytes", ctypes.c_double),
                ("mg_cycles", ctypes.c_int64), ("mg_ms", ctypes.c_double),
                ("resid_launches", ctypes.c_int64), ("resid_ms", ctypes.c_double), ("resid_bytes", ctypes.c_double),
                ("mg0a_launches", ctypes.c_int64), ("mg0a_ms", ctypes.c_double), ("mg0a_bytes", ctypes.c_double)]


class QmsSrvDesc(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_double), ("max_resident", ctypes.c_int), ("device", ctypes.c_int)]


class QmsRequest(ctypes.Structure):
    _fields_ = [("xs", ctypes.c_int), ("ys", ctypes.c_int), ("zs", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
                ("nt", ctypes.c_int), ("tt", ctypes.c_int), ("slice_axis", ctypes.c_int),
                ("slice_index", ctypes.c_int), ("keep", ctypes.c_int), ("precision", ctypes.c_int),
                ("B", ctypes.c_double * 3), ("G", ctypes.c_double * 9), ("traj", (ctypes.c_double * 3) * 3),
                ("exc_kind", ctypes.c_int), ("exc_f", ctypes.c_double), ("exc_phase", ctypes.c_double),
                ("geom", ctypes.c_void_p), ("table", ctypes.c_void_p), ("nmat", ctypes.c_int),
                ("traj_kind", ctypes.c_int * 3), ("traj_table", ctypes.c_void_p * 3), ("traj_len", ctypes.c_int * 3)]


class QmsSrvResult(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("rc", ctypes.c_int), ("n_dims", ctypes.c_longlong),
                ("steps_done", ctypes.c_int), ("arrival_s", ctypes.c_double), ("admitted_s", ctypes.c_double),
                ("finished_s", ctypes.c_double), ("steady_s", ctypes.c_double), ("step_mean_s", ctypes.c_double),
                ("step_max_s", ctypes.c_double), ("n_slice_values", ctypes.c_longlong)]


class QmsSrvStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong), ("failed", ctypes.c_longlong),
                ("rejected", ctypes.c_longlong), ("step_p50_ms", ctypes.c_double), ("step_p99_ms", ctypes.c_double),
                ("request_p50_s", ctypes.c_double), ("request_p99_s", ctypes.c_double),
                ("queue_wait_p50_s", ctypes.c_double), ("queue_wait_p99_s", ctypes.c_double),
                ("dof_timesteps", ctypes.c_double), ("wall_s", ctypes.c_double), ("peak_bytes", ctypes.c_double),
                ("peak_resident", ctypes.c_int)]


# struct name in include/qms.h -> ctypes mirror (checked field by field by tests/test_capi_cpu.py)
STRUCTS = {"qms_desc": None, "qms_stats": None, "qms_profile": None, "qms_srv_desc": QmsSrvDesc,
           "qms_request": QmsRequest, "qms_srv_result": QmsSrvResult, "qms_srv_stats": QmsSrvStats}

QMS_SRV_QUEUED, QMS_SRV_RUNNING, QMS_SRV_DONE, QMS_SRV_FAILED, QMS_SRV_REJECTED = range(5)
QMS_KEEP_NONE, QMS_KEEP_SLICES = 0, 1
QMS_EXC_NONE, QMS_EXC_COS, QMS_EXC_SIN = 0, 1, 2
QMS_PREC_MIXED, QMS_PREC_FP64 = 0, 1
QMS_FIELD_CUBES, QMS_FIELD_SLICE = 0, 1
# qms_stats.status bits
QMS_STATUS_BAD_MATERIAL, QMS_STATUS_NAN, QMS_STATUS_NO_CONVERGENCE = 1, 2, 4
QMS_STATUS_BREAKDOWN, QMS_STATUS_TIMEOUT = 8, 16
ERRORS = {-1: "QMS_ERR_ARG", -2: "QMS_ERR_CUDA", -3: "QMS_ERR_NOMEM", -4: "QMS_ERR_STATE", -5: "QMS_ERR_CONVERGE"}

# (name, restype, argtypes) -- the full export table of include/qms.h
_VP = ctypes.c_void_p
_DP = ctypes.POINTER(ctypes.c_double)
_H = ctypes.c_void_p
SIGNATURES = [
    ("qms_default_desc", None, [ctypes.POINTER(QmsDesc), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    ("qms_device_bytes", ctypes.c_size_t, [ctypes.POINTER(QmsDesc)]),
    ("qms_n_dims", ctypes.c_int64, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("qms_csr_nnz", ctypes.c_int64, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("qms_create", ctypes.c_int, [ctypes.POINTER(QmsDesc), ctypes.POINTER(_H)]),
    ("qms_destroy", None, [_H]),
    ("qms_last_error", ctypes.c_char_p, [_H]),
    ("qms_set_materials", ctypes.c_int, [_H, _VP, _VP, ctypes.c_int]),
    ("qms_set_geometry_f64", ctypes.c_int, [_H, _VP, _VP, ctypes.c_int]),
    ("qms_steady", ctypes.c_int, [_H, _DP, _DP, _DP]),
    ("qms_step", ctypes.c_int, [_H, _DP, _DP, _DP]),
    ("qms_get_stats", ctypes.c_int, [_H, ctypes.POINTER(QmsStats)]),
    ("qms_wait_selftest", ctypes.c_int, [_H, ctypes.c_int, ctypes.POINTER(ctypes.c_uint)]),
    ("qms_get_fields", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP]),
    ("qms_get_fields_async", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, ctypes.c_int]),
    ("qms_fields_sync", ctypes.c_int, [_H, ctypes.c_int]),
    ("qms_pinned_alloc", ctypes.c_void_p, [ctypes.c_size_t]),
    ("qms_pinned_free", None, [ctypes.c_void_p]),
    ("qms_get_state", ctypes.c_int, [_H, _VP]),
    ("qms_get_rhs", ctypes.c_int, [_H, _VP]),
    ("qms_set_state", ctypes.c_int, [_H, _VP]),
    ("qms_assemble_csr", ctypes.c_int, [_H, ctypes.c_int, _DP, _DP, _DP, _VP, _VP, _VP, _VP, _VP]),
    ("qms_apply", ctypes.c_int, [_H, ctypes.c_int, _DP, ctypes.c_int, _VP, _VP]),
    ("qms_csr_spmv", ctypes.c_int, [_H, _VP, _VP, _VP, _VP, _VP]),
    ("qms_residual_norm", ctypes.c_int, [_H, ctypes.c_int, _DP, _DP]),
    ("qms_profile_enable", ctypes.c_int, [_H, ctypes.c_int]),
    ("qms_get_profile", ctypes.c_int, [_H, ctypes.POINTER(QmsProfile)]),
    ("qms_get_stream", ctypes.c_void_p, [_H]),
    ("qms_residual_noalloc", ctypes.c_int, [ctypes.c_int] * 3 + [ctypes.c_double] * 4 + [ctypes.c_int, _DP, _VP, _VP,
                                                                                      ctypes.c_int, _VP, _VP, _VP,
                                                                                      _VP, _VP]),
    ("qms_residual_noalloc_fits", ctypes.c_int, [ctypes.c_int] * 3),
    ("qms_srv_create", ctypes.c_int, [ctypes.POINTER(QmsSrvDesc), ctypes.POINTER(_H)]),
    ("qms_srv_submit", ctypes.c_int, [_H, ctypes.POINTER(QmsRequest), ctypes.POINTER(ctypes.c_longlong)]),
    ("qms_srv_poll", ctypes.c_int, [_H, ctypes.c_longlong, ctypes.POINTER(QmsSrvResult)]),
    ("qms_srv_wait", ctypes.c_int, [_H, ctypes.c_longlong, ctypes.POINTER(QmsSrvResult)]),
    ("qms_srv_slices", ctypes.c_longlong, [_H, ctypes.c_longlong, _VP, ctypes.c_longlong]),
    ("qms_srv_error", ctypes.c_char_p, [_H, ctypes.c_longlong]),
    ("qms_srv_stats_get", ctypes.c_int, [_H, ctypes.POINTER(QmsSrvStats)]),
    ("qms_srv_destroy", None, [_H]),
    ("qms_srv_velocities", ctypes.c_int, [ctypes.POINTER(QmsRequest), ctypes.c_int, _VP]),
]
STRUCTS.update({"qms_desc": QmsDesc, "qms_stats": QmsStats, "qms_profile": QmsProfile})


def lib_path() -> str:
    return LIB


def load():
    """Load libqms_gb300.so (raises QMSLibraryError when it was not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB):
                raise QMSLibraryError(f"{LIB} is missing; build it with `python -m alpineqms_gb300.build`")
            L = ctypes.CDLL(LIB)
            for name, res, args in SIGNATURES:
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(rc: int, handle=None, what: str = ""):
    if rc == 0:
        return
    L = load()
    msg = L.qms_last_error(handle)
    msg = msg.decode() if msg else ""
    raise QMSError(rc, f"{what}: {ERRORS.get(rc, rc)}: {msg}")


class QMSError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def dvec(values):
    arr = (ctypes.c_double * len(values))(*[float(v) for v in values])
    return arr
