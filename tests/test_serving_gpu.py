"""Serving on the GPU: a request's result is bit-identical alone and in a mix of
concurrently resident solves (fixed-order reductions, independent streams)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _req(seed, shape, nt=4):
    from alpineqms_gb300 import workloads
    from alpineqms_gb300.serving import SolveRequest
    rng = np.random.default_rng(seed)
    inp, geom = workloads.serving_request(rng, sizes=(shape,), nt=nt)
    return SolveRequest(inp, geom, keep_fields="slice")


def test_alone_vs_mix_bit_identical():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from alpineqms_gb300.serving import Backend, QMSServer
    target = _req(11, (24, 24, 24))
    alone = QMSServer(budget_bytes=8 << 30, max_resident=1, backend=Backend()).serve([target])[0]
    assert alone.status == "ok", alone.error
    mix = [_req(12, (32, 32, 32)), _req(11, (24, 24, 24)), _req(13, (20, 28, 24)), _req(14, (28, 20, 16))]
    res = QMSServer(budget_bytes=8 << 30, max_resident=4, backend=Backend()).serve(mix)
    assert all(r.status == "ok" for r in res), [r.error for r in res]
    again = res[1]
    assert len(again.slices) == len(alone.slices) == 5
    for a, b in zip(alone.slices, again.slices):
        assert np.array_equal(a, b)


def test_native_server_matches_python_backend():
    """The native serving object and the Python scheduler run the same call sequence on
    the library: a request's slice records are bit-identical through either, alone and
    in a mix."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from alpineqms_gb300.serving import Backend, NativeServer, QMSServer
    ref = QMSServer(budget_bytes=8 << 30, max_resident=1, backend=Backend()).serve([_req(21, (24, 20, 16))])[0]
    assert ref.status == "ok", ref.error
    with NativeServer(budget_bytes=8 << 30, max_resident=3) as srv:
        res = srv.serve([_req(22, (20, 20, 20)), _req(21, (24, 20, 16)), _req(23, (16, 24, 20))])
        st = srv.stats()
    assert all(r.status == "ok" for r in res), [r.error for r in res]
    assert len(res[1].slices) == len(ref.slices) == 5
    for a, b in zip(res[1].slices, ref.slices):
        assert np.array_equal(a, b)
    assert st["completed"] == 3 and st["peak_resident"] >= 1
