"""Failure detection on the GPU without a GPU fault.

Every TMA-staged kernel waits for its tile copies with a bounded poll of an
mbarrier (mbar_wait_n in qms_tma.cuh): when a copy never lands, the wait
gives up, the kernel sets QMS_STATUS_TIMEOUT and returns, and the host reads
the status word.  qms_wait_selftest makes that wait run out on purpose -- one
CTA waits on a barrier that nothing completes and no copy targets, for a few
polls -- so the test checks the reported status and that the same handle then
solves normally.  Nothing here faults, traps or hangs the device.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_bounded_wait_reports_timeout_and_handle_recovers():
    from alpineqms_gb300 import _lib
    from alpineqms_gb300.solver import QMSSolver, default_desc
    xs = ys = zs = 12
    h = 1e-3
    geom = np.zeros((xs, ys, zs))
    geom[4:8, 4:8, 5:7] = 1
    props = np.array([[1, 1, 1, 1, 5.8e7, 5.8e7, 5.8e7]], np.float64)
    s = QMSSolver(default_desc(xs, ys, zs, h, h, h, 1e-5))
    s.set_geometry_f64(geom.flatten(order="F"), props)
    L = _lib.load()
    for spins in (1, 64):
        st = ctypes.c_uint(0)
        rc = L.qms_wait_selftest(s.h, spins, ctypes.byref(st))
        assert rc == 0
        assert st.value & _lib.QMS_STATUS_TIMEOUT
        assert s.stats()["status"] & _lib.QMS_STATUS_TIMEOUT
    # out-of-range bounds are refused before any launch
    assert L.qms_wait_selftest(s.h, 0, None) == -1
    assert L.qms_wait_selftest(s.h, (1 << 20) + 1, None) == -1
    # the handle and its context are still usable: a normal solve runs and reports a clean status
    B, G = np.array([0.0, 0.0, 1e-3]), np.zeros(9)
    st0 = s.steady([0, 0, 0], B, G)
    assert st0["status"] == 0 and st0["r"] <= 2e-13
    st1 = s.step([0, 0, 0], B, G)
    assert st1["status"] == 0 and st1["r"] <= 2e-13
    assert np.isfinite(s.get_state()).all()
    s.close()
