"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and the built engine library; the
rest run on any machine (CPU oracle, host logic, C-ABI symbol checks).
"""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
for p in (str(ROOT), str(GOLDEN)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libgmes_gb300.so")


def load_golden(name):
    arrays = dict(np.load(GOLDEN / f"{name}.npz"))
    meta = json.loads((GOLDEN / f"{name}.json").read_text())
    return arrays, meta


def checksum(a):
    a = np.asarray(a)
    if np.iscomplexobj(a):
        return [complex(np.sum(a)).real, complex(np.sum(a)).imag,
                float(np.sum(np.abs(a) ** 2)), float(np.max(np.abs(a)))]
    a = np.asarray(a, np.float64)
    return [float(np.sum(a)), float(np.sum(a * a)), float(np.max(np.abs(a)))]


def rel_l2(a, b):
    """Relative L2 error of a against reference b (0 when both are zero)."""
    a = np.asarray(a)
    b = np.asarray(b)
    if not (np.iscomplexobj(a) or np.iscomplexobj(b)):
        a = a.astype(np.float64)
        b = b.astype(np.float64)
    nb = np.linalg.norm(b)
    d = np.linalg.norm(a - b)
    return d / nb if nb > 0 else d


@pytest.fixture(scope="session")
def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
