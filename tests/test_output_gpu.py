"""The asynchronous field output (qms_get_fields_async / qms_fields_sync, pinned host buffers)
gives exactly what the synchronous qms_get_fields gives, step after step, while the next step
already runs; and the drop-in runner, which dumps through it, writes records identical to
ones written from the synchronous path (3D/QMS_3D.f90:2274-2300 cadence: slice every tt
steps, cubes every step)."""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _case(xs=18, ys=14, zs=12):
    geom = np.zeros((xs, ys, zs))
    geom[5:12, 4:10, 4:8] = 1
    props = np.array([[1, 1, 1, 1, 3.5e7, 3.5e7, 3.5e7]], np.float64)
    return geom.flatten(order="F"), props


def test_async_fields_match_sync_over_steps():
    from alpineqms_gb300._lib import QMS_FIELD_CUBES, QMS_FIELD_SLICE
    from alpineqms_gb300.solver import PinnedBuffer, QMSSolver, default_desc
    xs, ys, zs, h = 18, 14, 12, 1e-3
    geom, props = _case(xs, ys, zs)
    s = QMSSolver(default_desc(xs, ys, zs, h, h, h, 1e-5))
    s.set_geometry_f64(geom, props)
    B, G = np.array([0.0, 0.0, 1e-2]), np.array([-0.05, 0, 0, 0, -0.05, 0, 0, 0, 0.1])
    s.steady([0, 0, 0], B, G)
    n1, n2 = s.slice_shape("y")
    bs = [PinnedBuffer(3 * n1 * n2) for _ in range(2)]
    bc = [PinnedBuffer(3 * xs * ys * zs) for _ in range(2)]
    pending = []
    for k in range(6):
        s.step([-5.0, 0, 0], B * (1 + 0.1 * k), G)
        # the synchronous result of this step, then the same through the async path
        want_s = np.concatenate([a.ravel(order="F") for a in s.slices("y", 7)])
        want_c = np.concatenate([a.ravel(order="F") for a in s.fields()])
        s.fields_async(QMS_FIELD_SLICE, "y", 7, bs[k % 2], k % 2)
        s.fields_async(QMS_FIELD_CUBES, "x", 1, bc[k % 2], 2 + k % 2)
        pending.append((k % 2, want_s, want_c))
        if len(pending) == 2:      # check the previous step's copies after the next step started
            slot, ws, wc = pending.pop(0)
            s.fields_sync(slot)
            s.fields_sync(2 + slot)
            assert np.array_equal(bs[slot].array, ws)
            assert np.array_equal(bc[slot].array, wc)
    for slot, ws, wc in pending:
        s.fields_sync(slot)
        s.fields_sync(2 + slot)
        assert np.array_equal(bs[slot].array, ws)
        assert np.array_equal(bc[slot].array, wc)
    with pytest.raises(Exception):
        s.fields_async(QMS_FIELD_SLICE, "y", 7, bs[0], 4)          # slots 0..3
    for b in bs + bc:
        b.close()
    s.close()


def test_dropin_async_dumps_equal_sync_records(tmp_path):
    from alpineqms_gb300 import qms3d, workloads
    from alpineqms_gb300.records import DumpWriter, read_records
    from alpineqms_gb300.solver import QMSSolver, default_desc
    from alpineqms_gb300.trajectory import VelocitySchedule, scaled_field
    inp, geom = workloads.moving_plate(24, nt=5, plate=(16, 16, 3))
    inp = dataclasses.replace(inp, save_all="yes", tt=2)
    d_async = tmp_path / "async"
    workloads.write_case(str(d_async), inp, geom)
    qms3d.run(str(d_async / "inputs.txt"), workdir=str(d_async), log=lambda *a: None)
    # the same run dumped synchronously
    d_sync = tmp_path / "sync"
    d_sync.mkdir()
    s = QMSSolver(default_desc(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, inp.dt))
    s.set_geometry_f64(geom, inp.props_table())
    w = DumpWriter(inp, str(d_sync))
    sched = VelocitySchedule(inp.traj, inp.dt)
    for k in range(inp.nt + 1):
        B, G = scaled_field(inp.B, inp.G, inp.excitation, k * inp.dt)
        if k == 0:
            s.steady(sched.steady(), B, G)
        else:
            s.step(sched.step(k), B, G)
        if w.wants_slice(k):
            w.write_slice(s.slices(inp.slice_axis, inp.slice_index))
        if inp.save_all_fields:
            w.write_cube(s.fields())
    w.close()
    s.close()
    names = ["Hx.bin", "Hy.bin", "Hz.bin"] + (["Hx_all.bin", "Hy_all.bin", "Hz_all.bin"] if inp.save_all_fields else [])
    for nm in names:
        a, b = read_records(str(d_async / nm)), read_records(str(d_sync / nm))
        assert len(a) == len(b) and all(np.array_equal(x, y) for x, y in zip(a, b)), nm
