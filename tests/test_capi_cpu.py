"""C-ABI checks that need no GPU: the library loads, exports every function
include/qms.h declares, and its host-only size functions agree with the oracle."""
import ctypes
import os
import re

import pytest

import qms_oracle as o
from conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "qms.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qms_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from alpineqms_gb300 import build as b, _lib
    b.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = header_functions()
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n


def test_binding_table_matches_header():
    from alpineqms_gb300 import _lib
    bound = {s[0] for s in _lib.SIGNATURES}
    assert bound == set(header_functions())


@pytest.mark.parametrize("shape", [(6, 7, 8), (32, 32, 32), (17, 9, 23), (96, 96, 96), (128, 64, 32)])
def test_sizes_agree_with_oracle(lib, shape):
    n, nnz, _ = o.sizes(*shape)
    assert lib.qms_n_dims(*shape) == n
    assert lib.qms_csr_nnz(*shape) == nnz


def test_device_bytes_monotone(lib):
    from alpineqms_gb300._lib import QmsDesc
    d = QmsDesc()
    lib.qms_default_desc(ctypes.byref(d), 64, 64, 64, 1e-3, 1e-3, 1e-3, 1e-5)
    b64 = lib.qms_device_bytes(ctypes.byref(d))
    lib.qms_default_desc(ctypes.byref(d), 128, 128, 128, 1e-3, 1e-3, 1e-3, 1e-5)
    b128 = lib.qms_device_bytes(ctypes.byref(d))
    assert 7 * b64 < b128 < 9 * b64
    d.precision = 1
    assert lib.qms_device_bytes(ctypes.byref(d)) > b128


def test_create_without_gpu_fails_cleanly(lib):
    """No exception crosses the ABI: a failing create returns a code and a message."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from alpineqms_gb300._lib import QmsDesc
    d = QmsDesc()
    lib.qms_default_desc(ctypes.byref(d), 8, 8, 8, 1e-3, 1e-3, 1e-3, 1e-5)
    h = ctypes.c_void_p()
    rc = lib.qms_create(ctypes.byref(d), ctypes.byref(h))
    assert rc < 0 and not h.value
    assert lib.qms_last_error(None)


def test_struct_layouts_match_header(tmp_path):
    """Every struct of include/qms.h has the same size and field offsets in C (compiled
    here with gcc) as its ctypes mirror in alpineqms_gb300/_lib.py."""
    import shutil
    import subprocess
    from alpineqms_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "qms.h"', "int main(void) {"]
    for name, ct in _lib.STRUCTS.items():
        lines.append(f'printf("{name} size %zu\\n", sizeof({name}));')
        for fname, _ in ct._fields_:
            lines.append(f'printf("{name} {fname} %zu\\n", offsetof({name}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            a, b, c = ln.split()
            got[(a, b)] = int(c)
    for name, ct in _lib.STRUCTS.items():
        assert got[(name, "size")] == ctypes.sizeof(ct), name
        for fname, _ in ct._fields_:
            assert got[(name, fname)] == getattr(ct, fname).offset, (name, fname)


def test_default_descriptor(lib):
    """qms_default_desc (host-only) fills the documented defaults of the solver."""
    from alpineqms_gb300._lib import QmsDesc
    d = QmsDesc()
    lib.qms_default_desc(ctypes.byref(d), 64, 48, 32, 1e-3, 2e-3, 3e-3, 1e-5)
    assert (d.xs, d.ys, d.zs) == (64, 48, 32)
    assert (d.dx, d.dy, d.dz, d.dt) == (1e-3, 2e-3, 3e-3, 1e-5)
    assert d.tol == 2e-13 and d.gmres_m == 32 and d.max_outer == 60
    assert d.mg_sweeps == 3 and d.mg_omega == 0.85 and d.mg_alpha == 1.5
    assert d.mg_coupling == 1 and d.extrapolate == 3 and d.gm_first_extend == 0 and d.start_ls == 4


def test_noalloc_size_query(lib):
    """qms_residual_noalloc_fits (host arithmetic only) accepts grids whose operator tiles fit the
    no-allocation entry point's fixed scratch (32768 tiles of 32 x 8 x 16 nodes) and rejects
    larger ones; qms_residual_noalloc turns the same grids away before any launch."""
    def tiles(xs, ys, zs):
        return -(-(xs + 1) // 32) * -(-(ys + 1) // 8) * -(-(zs + 1) // 16)
    for shape in [(4, 4, 4), (32, 32, 32), (256, 256, 256), (512, 512, 256), (2048, 2048, 2048), (3, 8, 8),
                  (1000, 1000, 100)]:
        want = 1 if min(shape) >= 4 and tiles(*shape) <= 32768 else 0
        assert lib.qms_residual_noalloc_fits(*shape) == want, shape
    assert lib.qms_residual_noalloc_fits(512, 512, 256) == 1
    assert lib.qms_residual_noalloc_fits(2048, 2048, 2048) == 0
