import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libdesgpu.so")


def load_golden(name):
    path = os.path.join(HERE, "golden", f"{name}.npz")
    z = np.load(path)
    out = {}
    for k in z.files:
        if "/" in k:
            grp, key = k.split("/", 1)
            out.setdefault(grp, {})[key] = z[k]
        else:
            out[k] = z[k]
    return out


def state_from(group: dict) -> dict:
    from dynearthsol_gb300.capi import STATE_ARRAYS
    return {k: np.ascontiguousarray(group[k].copy()) for k in STATE_ARRAYS}


def rel_err(a, b):
    """max |a-b| normalised by max |b| (0 when both vanish)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max() if b.size else 0.0
    d = np.abs(a - b).max() if b.size else 0.0
    if scale == 0:
        return float(d)
    return float(d / scale)


@pytest.fixture(scope="session")
def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
