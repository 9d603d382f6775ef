"""Shared test setup.

Tests marked ``gpu`` need a CUDA device and the built library; everything else
runs on CPU (the oracle, the host-side reader/writer logic, the C-ABI export
table of the library, the serving scheduler and the multi-rank host logic).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ("aniso_accel", "static_block", "random_ramp")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libqms_gb300.so")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def golden():
    return {n: load_golden(n) for n in GOLDEN_CASES}
