"""Continuous-batching serving loop for QMS solves on one GPU.

A request is a whole solve: geometry (float64 material IDs), material table,
background field with optional AC excitation, frame trajectory, time step and
step count -- everything ``inputs.txt`` + ``geom.bin`` carry for the reference
program (3D/master.py:16-77).  The server

* admits requests in arrival order while the HBM budget and the slot limit
  allow, charging each its exact device footprint (``qms_device_bytes``:
  solution, multigrid hierarchy, Krylov workspace);
* keeps every admitted solve resident in HBM (its own qms_handle) and advances
  all resident solves concurrently: each runs on its own CUDA stream, driven
  by its own host thread (the ctypes calls release the GIL), so their kernels
  overlap on the device; a request that arrives while others are running is
  admitted as soon as memory and a slot free up, without waiting for the
  batch to drain;
* records per-step latency, queue wait and end-to-end latency per request,
  and the aggregate DOF-timesteps/s of the whole stream.

Every reduction in the library is a fixed-order block-partial sum, so a
request's result does not depend on what else is resident: alone and in a mix
it is bit-identical (tests/test_serving_gpu.py).
"""
from __future__ import annotations

import dataclasses
import heapq
import itertools
import queue
import threading
import time
from typing import Callable, Dict, List, Optional

import numpy as np


@dataclasses.dataclass
class SolveRequest:
    """One solve: the content of an inputs.txt + geom.bin pair."""
    inputs: object                 # alpineqms_gb300.inputs.QMSInputs
    geom: np.ndarray               # float64 material IDs, Fortran order
    arrival: float = 0.0           # offered arrival time (s, relative to server start)
    keep_fields: str = "slice"     # "slice" (the dump of every step), "final" or "none"
    request_id: int = -1


@dataclasses.dataclass
class SolveResult:
    request_id: int
    n_dims: int
    steps: int
    arrival: float
    admitted: float
    finished: float
    step_latency: List[float]      # seconds per transient step
    steady_latency: float
    slices: List[np.ndarray]       # per record: stacked (Hx, Hy, Hz) slice
    final_fields: Optional[List[np.ndarray]]
    status: str = "ok"
    error: str = ""

    @property
    def latency(self) -> float:
        return self.finished - self.arrival

    @property
    def queue_wait(self) -> float:
        return self.admitted - self.arrival


class Backend:
    """Creates and runs one solve.  The default backend drives libqms_gb300; tests
    substitute a host-only fake to exercise the scheduler without a GPU."""

    def footprint(self, req: SolveRequest) -> int:
        from .solver import default_desc, device_bytes
        i = req.inputs
        return device_bytes(default_desc(i.xs, i.ys, i.zs, i.dx, i.dy, i.dz, i.dt, precision=self.precision,
                                         device=self.device))

    def __init__(self, device: int = 0, precision: str = "mixed"):
        self.device = device
        self.precision = precision

    def run(self, req: SolveRequest, on_step: Callable[[int, float], None]) -> Dict:
        from .solver import QMSSolver, default_desc
        from .trajectory import VelocitySchedule, scaled_field
        i = req.inputs
        desc = default_desc(i.xs, i.ys, i.zs, i.dx, i.dy, i.dz, i.dt, precision=self.precision, device=self.device)
        slices, final = [], None
        with QMSSolver(desc) as s:
            s.set_geometry_f64(req.geom, i.props_table())
            sched = VelocitySchedule(i.traj, i.dt)
            B, G = scaled_field(i.B, i.G, i.excitation, 0.0)
            t0 = time.perf_counter()
            s.steady(sched.steady(), B, G)
            if req.keep_fields == "slice":
                slices.append(np.concatenate(s.slices(i.slice_axis, i.slice_index)).ravel())
            on_step(0, time.perf_counter() - t0)
            for n in range(1, i.nt + 1):
                t1 = time.perf_counter()
                B, G = scaled_field(i.B, i.G, i.excitation, n * i.dt)
                s.step(sched.step(n), B, G)
                if req.keep_fields == "slice" and n % i.tt == 0:
                    slices.append(np.concatenate(s.slices(i.slice_axis, i.slice_index)).ravel())
                on_step(n, time.perf_counter() - t1)
            if req.keep_fields == "final":
                final = [h.copy() for h in s.fields()]
            n_dims = s.n
        return {"n_dims": n_dims, "slices": slices, "final": final}


class QMSServer:
    """FIFO admission under an HBM budget and a slot limit; resident solves run concurrently."""

    def __init__(self, budget_bytes: int = 150 << 30, max_resident: int = 16, backend: Backend = None):
        self.budget = int(budget_bytes)
        self.max_resident = int(max_resident)
        self.backend = backend or Backend()
        self._pending: "queue.Queue[SolveRequest]" = queue.Queue()
        self._lock = threading.Condition()
        self._used = 0
        self._resident = 0
        self._results: Dict[int, SolveResult] = {}
        self._ids = itertools.count()
        self._t0 = None
        self._threads: List[threading.Thread] = []
        self.peak_resident = 0
        self.peak_bytes = 0

    # ------------------------------------------------------------------
    def now(self) -> float:
        return time.perf_counter() - self._t0

    def submit(self, req: SolveRequest) -> int:
        req.request_id = next(self._ids)
        if self._t0 is None:
            self._t0 = time.perf_counter()
        req.arrival = self.now()
        fp = self.backend.footprint(req)
        if fp > self.budget:
            self._results[req.request_id] = SolveResult(req.request_id, 0, 0, req.arrival, req.arrival, req.arrival,
                                                        [], 0.0, [], None, "rejected",
                                                        f"needs {fp} bytes, budget {self.budget}")
            return req.request_id
        req._footprint = fp
        self._pending.put(req)
        return req.request_id

    def _admit_loop(self, stop: threading.Event):
        while not (stop.is_set() and self._pending.empty()):
            try:
                req = self._pending.get(timeout=0.01)
            except queue.Empty:
                continue
            with self._lock:     # FIFO: the head waits until it fits (no overtaking)
                while self._used + req._footprint > self.budget or self._resident >= self.max_resident:
                    self._lock.wait(timeout=0.05)
                self._used += req._footprint
                self._resident += 1
                self.peak_resident = max(self.peak_resident, self._resident)
                self.peak_bytes = max(self.peak_bytes, self._used)
            admitted = self.now()
            th = threading.Thread(target=self._run_one, args=(req, admitted), daemon=True)
            th.start()
            self._threads.append(th)

    def _run_one(self, req: SolveRequest, admitted: float):
        steps: List[float] = []
        steady = [0.0]

        def on_step(n, dt):
            if n == 0:
                steady[0] = dt
            else:
                steps.append(dt)
        try:
            out = self.backend.run(req, on_step)
            res = SolveResult(req.request_id, out["n_dims"], len(steps), req.arrival, admitted, self.now(), steps,
                              steady[0], out["slices"], out["final"])
        except Exception as e:   # a failing solve is reported, the server keeps serving
            res = SolveResult(req.request_id, 0, len(steps), req.arrival, admitted, self.now(), steps, steady[0],
                              [], None, "failed", repr(e))
        with self._lock:
            self._results[req.request_id] = res
            self._used -= req._footprint
            self._resident -= 1
            self._lock.notify_all()

    # ------------------------------------------------------------------
    def serve(self, requests: List[SolveRequest], gaps: Optional[List[float]] = None) -> List[SolveResult]:
        """Offer `requests` with the given inter-arrival gaps (s) and wait for all of them."""
        self._t0 = time.perf_counter()
        stop = threading.Event()
        adm = threading.Thread(target=self._admit_loop, args=(stop,), daemon=True)
        adm.start()
        t_next = 0.0
        for q, req in enumerate(requests):
            if gaps is not None:
                t_next += gaps[q]
                delay = t_next - self.now()
                if delay > 0:
                    time.sleep(delay)
            self.submit(req)
        stop.set()
        adm.join()
        for th in list(self._threads):
            th.join()
        return [self._results[k] for k in sorted(self._results)]


def request_struct(i, geom, keep_slices: bool, precision: int):
    """The qms_request of one solve (include/qms.h) and the arrays its pointers borrow: the
    caller keeps the second value alive until the request is submitted (the server copies
    them at submit)."""
    from . import _lib as lib
    r = lib.QmsRequest()
    r.xs, r.ys, r.zs = i.xs, i.ys, i.zs
    r.dx, r.dy, r.dz, r.dt = i.dx, i.dy, i.dz, i.dt
    r.nt, r.tt = i.nt, i.tt
    r.slice_axis = {"x": 0, "y": 1, "z": 2}[i.slice_axis]
    r.slice_index = i.slice_index
    r.keep = lib.QMS_KEEP_SLICES if keep_slices else lib.QMS_KEEP_NONE
    r.precision = precision
    for c in range(3):
        r.B[c] = float(i.B[c])
    for c, g in enumerate(np.asarray(i.G, dtype=np.float64).reshape(9)):
        r.G[c] = float(g)
    keep = []
    for d, t in enumerate(i.traj):
        r.traj_kind[d] = int(t.kind)
        if t.kind == 2:
            r.traj[d][0], r.traj[d][1], r.traj[d][2] = float(t.amp), float(t.freq), float(t.phase)
        elif t.kind == 3:
            tab = np.ascontiguousarray(t.table, dtype=np.float64)
            keep.append(tab)
            r.traj_table[d], r.traj_len[d] = tab.ctypes.data, tab.size
        else:
            r.traj[d][0], r.traj[d][1], r.traj[d][2] = float(t.v0), float(t.accel), float(t.n_accel)
    if i.excitation is None:
        r.exc_kind = lib.QMS_EXC_NONE
    else:
        kind, f, ph = i.excitation
        r.exc_kind = lib.QMS_EXC_COS if kind == "cos" else lib.QMS_EXC_SIN
        r.exc_f, r.exc_phase = float(f), float(ph)
    if geom is not None:
        g = np.ascontiguousarray(geom, dtype=np.float64)
        table = np.ascontiguousarray(i.props_table(), dtype=np.float64)
        keep += [g, table]
        r.geom, r.table, r.nmat = g.ctypes.data, table.ctypes.data, table.shape[0]
    return r, keep


class NativeServer:
    """The serving object of libqms_gb300 (``qms_srv_*`` in include/qms.h): the same FIFO
    admission under an HBM budget and slot limit as QMSServer, with the admission and
    the per-request solves run by native threads.  Requests and results use the same
    SolveRequest / SolveResult types; a result's slice records have the layout of
    Backend.run."""

    def __init__(self, budget_bytes: int = 150 << 30, max_resident: int = 16, device: int = 0,
                 precision: str = "mixed"):
        import ctypes
        from . import _lib
        self._ct = ctypes
        self._lib = _lib
        self.L = _lib.load()
        self.precision = _lib.QMS_PREC_FP64 if precision == "fp64" else _lib.QMS_PREC_MIXED
        d = _lib.QmsSrvDesc(float(budget_bytes), int(max_resident), int(device))
        self.h = ctypes.c_void_p()
        rc = self.L.qms_srv_create(ctypes.byref(d), ctypes.byref(self.h))
        if rc:
            raise _lib.QMSError(rc, f"qms_srv_create: {_lib.ERRORS.get(rc, rc)}")
        self._reqs: Dict[int, SolveRequest] = {}

    def submit(self, req: SolveRequest) -> int:
        ct, lib = self._ct, self._lib
        r, keep_alive = request_struct(req.inputs, req.geom, req.keep_fields == "slice", self.precision)
        rid = ct.c_longlong()
        rc = self.L.qms_srv_submit(self.h, ct.byref(r), ct.byref(rid))   # copies geom and table
        if rc:
            raise lib.QMSError(rc, f"qms_srv_submit: {lib.ERRORS.get(rc, rc)}")
        req.request_id = int(rid.value)
        self._reqs[req.request_id] = req
        return req.request_id

    def wait(self, rid: int) -> SolveResult:
        ct, lib = self._ct, self._lib
        out = lib.QmsSrvResult()
        self.L.qms_srv_wait(self.h, rid, ct.byref(out))
        req = self._reqs[rid]
        i = req.inputs
        slices = []
        if out.n_slice_values > 0:
            buf = np.empty(out.n_slice_values, np.float64)
            self.L.qms_srv_slices(self.h, rid, buf.ctypes.data, buf.size)
            n1, n2 = i.slice_shape()
            m = n1 * n2
            for rec in buf.reshape(-1, 3 * m):
                slices.append(np.concatenate([rec[q * m:(q + 1) * m].reshape((n1, n2), order="F")
                                              for q in range(3)]).ravel())
        status = {lib.QMS_SRV_DONE: "ok", lib.QMS_SRV_FAILED: "failed", lib.QMS_SRV_REJECTED: "rejected"}.get(
            out.state, "unknown")
        err = self.L.qms_srv_error(self.h, rid)
        return SolveResult(rid, int(out.n_dims), int(out.steps_done), out.arrival_s, out.admitted_s, out.finished_s,
                           [out.step_mean_s] * int(out.steps_done), out.steady_s, slices, None, status,
                           err.decode() if err else "")

    def serve(self, requests: List[SolveRequest], gaps: Optional[List[float]] = None) -> List[SolveResult]:
        t0 = time.perf_counter()
        t_next = 0.0
        ids = []
        for q, req in enumerate(requests):
            if gaps is not None:
                t_next += gaps[q]
                delay = t_next - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
            ids.append(self.submit(req))
        return [self.wait(r) for r in ids]

    def stats(self) -> Dict:
        ct, lib = self._ct, self._lib
        st = lib.QmsSrvStats()
        self.L.qms_srv_stats_get(self.h, ct.byref(st))
        out = {k: getattr(st, k) for k, _ in lib.QmsSrvStats._fields_}
        out["dof_timesteps_per_s"] = st.dof_timesteps / st.wall_s if st.wall_s > 0 else None
        return out

    def close(self):
        if self.h:
            self.L.qms_srv_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def latency_report(results: List[SolveResult], wall: float) -> Dict:
    ok = [r for r in results if r.status == "ok"]
    steps = np.array([x for r in ok for x in r.step_latency]) if ok else np.zeros(0)
    req = np.array([r.latency for r in ok]) if ok else np.zeros(0)
    waits = np.array([r.queue_wait for r in ok]) if ok else np.zeros(0)
    dof_steps = sum(r.n_dims * r.steps for r in ok)

    def pct(a, p):
        return float(np.percentile(a, p)) if a.size else None
    errors: Dict[str, int] = {}
    for r in results:
        if r.status != "ok":
            key = r.error[:200]
            errors[key] = errors.get(key, 0) + 1
    return {"requests": len(results), "completed": len(ok),
            "failed": sum(r.status == "failed" for r in results),
            "rejected": sum(r.status == "rejected" for r in results),
            "errors": errors,
            "step_p50_ms": 1e3 * pct(steps, 50) if steps.size else None,
            "step_p99_ms": 1e3 * pct(steps, 99) if steps.size else None,
            "request_p50_s": pct(req, 50), "request_p99_s": pct(req, 99),
            "queue_wait_p50_s": pct(waits, 50), "queue_wait_p99_s": pct(waits, 99),
            "dof_timesteps_per_s": dof_steps / wall if wall > 0 else None, "wall_s": wall}


def poisson_stream(n: int, mean_gap: float, seed: int = 4, nt: int = 50, sizes=None):
    """The seeded serving workload: n requests with exponential gaps (mean `mean_gap` s)."""
    from . import workloads
    rng = np.random.default_rng(np.random.PCG64(seed))
    reqs, gaps = [], []
    for _ in range(n):
        inp, geom = workloads.serving_request(rng, nt=nt, **({"sizes": sizes} if sizes else {}))
        reqs.append(SolveRequest(inp, geom, keep_fields="none"))
        gaps.append(float(rng.exponential(mean_gap)))
    return reqs, gaps


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="serve a seeded Poisson stream of QMS solves")
    ap.add_argument("--requests", type=int, default=512)
    ap.add_argument("--mean-gap", type=float, default=0.05)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--max-resident", type=int, default=16)
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--scheduler", default="native", choices=["native", "python"])
    a = ap.parse_args(argv)
    reqs, gaps = poisson_stream(a.requests, a.mean_gap, nt=a.steps)
    budget = int(a.budget_gb * (1 << 30))
    t0 = time.perf_counter()
    if a.scheduler == "native":
        with NativeServer(budget, a.max_resident, precision=a.precision) as srv:
            res = srv.serve(reqs, gaps)
            wall = time.perf_counter() - t0
            rep = latency_report(res, wall)
            st = srv.stats()
            # per-step percentiles from the native per-step timings
            rep.update({"step_p50_ms": st["step_p50_ms"], "step_p99_ms": st["step_p99_ms"],
                        "peak_resident": st["peak_resident"], "peak_bytes": st["peak_bytes"]})
    else:
        srv = QMSServer(budget, a.max_resident, Backend(precision=a.precision))
        res = srv.serve(reqs, gaps)
        wall = time.perf_counter() - t0
        rep = latency_report(res, wall)
        rep.update({"peak_resident": srv.peak_resident, "peak_bytes": srv.peak_bytes})
    rep.update({"scheduler": a.scheduler, "mean_gap_s": a.mean_gap, "steps_per_request": a.steps,
                "precision": a.precision})
    print(json.dumps(rep))


if __name__ == "__main__":
    main()
