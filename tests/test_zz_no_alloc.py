"""qms_residual_noalloc: the residual entry point for callers that cannot allocate.

Callers such as an allocator-free real-time loop, or a process whose device
memory belongs to another runtime's pool, cannot call cudaMalloc and cannot
create a qms_handle.  qms_residual_noalloc takes
only their own device buffers and keeps its scratch in fixed-size static
device arrays.  This test calls it through the C-ABI twice in a row and checks
each result against qms_residual_norm (the handle-based entry point) on the
same state and right-hand side.

The file is named so that pytest collects it last; it also passes alone in a
fresh process.  (The size limit of its fixed scratch is checked on the CPU
through qms_residual_noalloc_fits in tests/test_capi_cpu.py.)
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc_fn():
    from alpineqms_gb300 import _lib
    L = _lib.load()
    fn = L.qms_residual_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 4 + [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                                 ctypes.c_void_p, ctypes.c_void_p]
    return fn


def test_noalloc_residual_matches_handle_entry_point():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from alpineqms_gb300._lib import dvec
    from alpineqms_gb300.inputs import Material, QMSInputs, Trajectory, material_index
    from alpineqms_gb300.solver import QMSSolver, default_desc

    xs, ys, zs, h, dt = 14, 12, 10, 1e-3, 1e-5
    geom = np.zeros((xs, ys, zs))
    geom[4:10, 3:9, 3:7] = 1
    geom[6:8, 5:7, 4:6] = 2
    table = np.array([[1, 1, 1, 1, 3.5e7, 3.5e7, 3.5e7], [2, 50, 50, 50, 2e6, 2e6, 2e6]], np.float64)
    v = [-3.0, 0.0, 1.0]
    B = np.array([1e-3, 2e-3, 5e-3])
    G = np.array([-0.05, 0, 0, 0, -0.05, 0, 0, 0, 0.1])

    s = QMSSolver(default_desc(xs, ys, zs, h, h, h, dt))
    s.set_geometry_f64(geom.flatten(order="F"), table)
    s.steady([0.0, 0.0, 0.0], B, G)
    x0 = s.get_state()
    s.step(v, B, G)
    x1 = s.get_state()
    n = s.n

    # right-hand side of that step on the device (bit-identical to the one the step used)
    nnz = int(s.L.qms_csr_nnz(xs, ys, zs))
    t_ia = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    t_ja = torch.empty(nnz, dtype=torch.int32, device="cuda")
    t_a = torch.empty(nnz, dtype=torch.float64, device="cuda")
    t_b = torch.empty(n, dtype=torch.float64, device="cuda")
    t_x0 = torch.from_numpy(x0).cuda()
    s.assemble_csr(True, v, B, G, t_x0.data_ptr(), t_ia.data_ptr(), t_ja.data_ptr(), t_a.data_ptr(), t_b.data_ptr())

    # material slots as the caller's own device buffer
    inp = QMSInputs(xs, ys, zs, h, h, h, dt, 1, 1, "z", 1, "no", tuple(B), ((0, 0, 0),) * 3,
                    tuple(Trajectory(1, 0.0, 0.0, 0) for _ in range(3)),
                    [Material(r[0], tuple(r[1:4]), tuple(r[4:7])) for r in table], "geom.bin")
    slots = material_index(geom.flatten(order="F"), inp)
    t_slots = torch.from_numpy(slots).cuda()
    rows6 = np.ascontiguousarray(table[:, 1:7])

    fn = _noalloc_fn()
    t_r = torch.empty(n, dtype=torch.float64, device="cuda")
    t_sums = torch.empty(4, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    for x in (x1, x0):                  # two calls in a row, different states
        s.set_state(x)
        rel_handle = s.residual_norm(True, v)
        t_x = torch.from_numpy(x).cuda()
        torch.cuda.synchronize()
        rc = fn(xs, ys, zs, h, h, h, dt, 1, dvec(v), t_slots.data_ptr(), rows6.ctypes.data, rows6.shape[0],
                t_x.data_ptr(), t_b.data_ptr(), t_r.data_ptr(), t_sums.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        sums = t_sums.cpu().numpy()
        rel = np.sqrt(sums[0] + sums[1]) / np.sqrt(sums[2] + sums[3])
        assert np.isfinite(rel) and rel_handle > 0
        assert abs(rel - rel_handle) <= 1e-12 * rel_handle, (rel, rel_handle)
        # the returned residual vector is consistent with the returned sums
        r = t_r.cpu().numpy()
        assert abs(np.sqrt(np.dot(r, r)) - np.sqrt(sums[0] + sums[1])) <= 1e-12 * np.sqrt(sums[0] + sums[1])
    s.close()
