import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle"), GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


def pytest_collection_modifyitems(config, items):
    # the GPU tests need the CUDA library; build it once before they run
    if any("gpu" in item.keywords for item in items):
        try:
            from plbpd_gb300 import build as _b
            _b.build()
        except Exception:
            pass


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def load_npz(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def assert_bitexact(got, want, what=""):
    g, w = bits(got), bits(want)
    assert g.shape == w.shape, f"{what}: shape {g.shape} != {w.shape}"
    bad = np.argwhere(g != w)
    if bad.size:
        i = tuple(bad[0])
        raise AssertionError(f"{what}: {len(bad)} of {g.size} values differ; first at {i}: "
                             f"got {np.asarray(got)[i]!r} want {np.asarray(want)[i]!r}")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
