"""Serving scheduler on the host (no GPU): admission under the HBM budget and the
slot limit, FIFO order, continuous admission while others run, failure isolation."""
import threading
import time

import numpy as np
import pytest

from alpineqms_gb300.serving import Backend, QMSServer, SolveRequest, latency_report


class FakeInputs:
    def __init__(self, nt, size):
        self.nt, self.size = nt, size


class FakeBackend(Backend):
    """Footprint = size; each step sleeps; records concurrency."""

    def __init__(self, step_s=0.01, fail_ids=()):
        self.step_s = step_s
        self.fail_ids = set(fail_ids)
        self.lock = threading.Lock()
        self.active = 0
        self.max_active = 0
        self.order = []

    def footprint(self, req):
        return req.inputs.size

    def run(self, req, on_step):
        with self.lock:
            self.active += 1
            self.max_active = max(self.max_active, self.active)
            self.order.append(req.request_id)
        try:
            if req.request_id in self.fail_ids:
                raise RuntimeError("solver failure")
            on_step(0, 0.0)
            for n in range(1, req.inputs.nt + 1):
                time.sleep(self.step_s)
                on_step(n, self.step_s)
            return {"n_dims": 1000, "slices": [], "final": None}
        finally:
            with self.lock:
                self.active -= 1


def reqs(sizes, nt=3):
    return [SolveRequest(FakeInputs(nt, s), np.zeros(1)) for s in sizes]


def test_budget_and_slots_respected():
    be = FakeBackend()
    srv = QMSServer(budget_bytes=100, max_resident=3, backend=be)
    res = srv.serve(reqs([40, 40, 40, 30, 20, 60, 10]))
    assert all(r.status == "ok" for r in res)
    assert srv.peak_bytes <= 100
    assert srv.peak_resident <= 3
    assert be.max_active <= 3
    assert be.order == sorted(be.order)          # FIFO admission


def test_oversize_request_rejected_others_served():
    srv = QMSServer(budget_bytes=50, max_resident=4, backend=FakeBackend())
    res = srv.serve(reqs([10, 80, 20]))
    assert [r.status for r in res] == ["ok", "rejected", "ok"]


def test_continuous_admission_while_running():
    """A request arriving while a long one runs starts before the long one ends."""
    be = FakeBackend(step_s=0.02)
    srv = QMSServer(budget_bytes=100, max_resident=4, backend=be)
    long_req = SolveRequest(FakeInputs(20, 50), np.zeros(1))
    short = SolveRequest(FakeInputs(2, 40), np.zeros(1))
    res = srv.serve([long_req, short], gaps=[0.0, 0.05])
    r_long, r_short = res
    assert r_short.admitted < r_long.finished
    assert r_short.finished < r_long.finished
    assert be.max_active == 2


def test_failure_is_isolated():
    be = FakeBackend(fail_ids={1})
    srv = QMSServer(budget_bytes=100, max_resident=2, backend=be)
    res = srv.serve(reqs([10, 10, 10]))
    assert [r.status for r in res] == ["ok", "failed", "ok"]
    assert "solver failure" in res[1].error
    rep = latency_report(res, wall=1.0)
    assert rep["completed"] == 2 and rep["failed"] == 1
    assert rep["step_p50_ms"] == pytest.approx(10.0)


def test_native_scheduler_without_gpu():
    """The native serving object (qms_srv_*) on a host without a GPU: every admitted
    request ends FAILED with the create error (none hangs), a request larger than the
    whole budget is REJECTED at submit, the stats count both, and destroy returns."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("runs where qms_create cannot succeed")
    from alpineqms_gb300 import build, workloads
    from alpineqms_gb300.serving import NativeServer
    build.build()
    rng = np.random.default_rng(3)
    small = [workloads.serving_request(rng, sizes=((16, 16, 16),), nt=2) for _ in range(5)]
    big = workloads.serving_request(rng, sizes=((128, 128, 128),), nt=2)
    from alpineqms_gb300.solver import default_desc, device_bytes
    i0 = small[0][0]
    fp_small = device_bytes(default_desc(i0.xs, i0.ys, i0.zs, i0.dx, i0.dy, i0.dz, i0.dt))
    with NativeServer(budget_bytes=3 * fp_small, max_resident=2) as srv:
        reqs = [SolveRequest(inp, geom) for inp, geom in small] + [SolveRequest(*big)]
        res = srv.serve(reqs)
        st = srv.stats()
    assert [r.status for r in res] == ["failed"] * 5 + ["rejected"]
    assert all("qms_create" in r.error for r in res[:5])
    assert st["submitted"] == 6 and st["failed"] == 5 and st["rejected"] == 1 and st["completed"] == 0
    assert 1 <= st["peak_resident"] <= 2
    assert st["peak_bytes"] <= 3 * fp_small
    # admission in arrival order
    adm = [r.admitted for r in res[:5]]
    assert adm == sorted(adm)
