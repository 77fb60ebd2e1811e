import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the native kernels")


def _has_cuda():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_cuda():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


class Golden:
    """Golden vectors produced by tests/golden/make_golden.py from the reference."""

    def __init__(self):
        self.z = np.load(os.path.join(GOLDEN_DIR, "golden.npz"))
        with open(os.path.join(GOLDEN_DIR, "manifest.json")) as f:
            self.manifest = json.load(f)

    def case(self, family, name):
        pre = "%s/%s/" % (family, name)
        return {k[len(pre):]: self.z[k] for k in self.z.files if k.startswith(pre)}

    def cases(self, family):
        return [m for m in self.manifest[family]]


@pytest.fixture(scope="session")
def golden():
    return Golden()


def obs_dict(n, kind, q0, q1, w):
    """Observable dict in the reference's format from term arrays."""
    d = {}
    for key, k in (("x", 0), ("y", 1), ("z", 2)):
        sel = kind == k
        if np.any(sel):
            arr = np.full(n, None)
            for q, v in zip(q0[sel], w[sel]):
                arr[int(q)] = float(v)
            d[key] = arr
    sel = kind == 3
    if np.any(sel):
        zz = np.full((n, n), None)
        for a, b, v in zip(q0[sel], q1[sel], w[sel]):
            zz[int(a), int(b)] = float(v)
        d["zz"] = zz
    return d


def rel_err(a, b):
    """Normwise relative error ||a - b||_inf / max(||b||_inf, tiny)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
