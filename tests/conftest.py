"""Shared pytest setup: markers, import paths, the GPU context fixture and data helpers."""

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "rstsr-showcase-hessian_gb300"))
sys.path.insert(0, str(REPO))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libcphf.so")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def built_lib():
    import cphf_gb300
    cphf_gb300.build()
    return cphf_gb300.load_library()


def load_golden(name):
    with np.load(GOLDEN / name) as z:
        return {k: z[k] for k in z.files}


def fp(x):
    """The reference's fingerprint ``sum_i cos(i) x_i`` over col-major order (tests/test_util.rs:60-62)."""
    flat = np.asarray(x).reshape(-1, order="F")
    return float(np.dot(np.cos(np.arange(flat.size)), flat))


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
