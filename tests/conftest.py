"""Shared test setup: import paths, the `gpu` marker, golden-fixture access
and builds of the oracle / engine libraries when they are missing."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_ROOT = os.path.join(ROOT, "magnus-dp_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG_ROOT, ORACLE_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 engine)")


def _ensure_built():
    lib = os.path.join(PKG_ROOT, "magnus_gb300", "libmagnus_gb300.so")
    if not os.path.exists(lib):
        subprocess.run(["make", "-s", "-j8", "-C", PKG_ROOT], check=True)
    if not os.path.exists(os.path.join(ORACLE_DIR, "_build", "libmagnus_oracle.so")):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


_ensure_built()


def load_cases(name):
    """Golden cases of tests/golden/<name>.npz as {case: {field: value}}."""
    data = np.load(os.path.join(GOLDEN, name))
    cases = {}
    for key in data.files:
        case, field = key.split("/", 1)
        v = data[key]
        cases.setdefault(case, {})[field] = v.item() if v.shape == () else v
    return cases


def rel(a, b):
    """Relative Frobenius distance ||a - b|| / ||b|| (complex-aware)."""
    a, b = np.asarray(a), np.asarray(b)
    t = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    a = a.astype(t)
    b = b.astype(t)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
