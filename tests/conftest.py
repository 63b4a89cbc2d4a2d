import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "chbrclf.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def chbrclf():
    from qmckl_sycl_gb300.systems import System

    return System.from_npz(GOLDEN)


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


def normwise_rel_err(got, ref, axis_comp=1):
    """max |got - ref| / max |ref|, per component (axis 1 of [P][5][n] arrays), maximised."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    if got.ndim == 3:
        scale = np.abs(ref).max(axis=(0, 2))
        diff = np.abs(got - ref).max(axis=(0, 2))
        return float((diff / np.maximum(scale, 1e-300)).max())
    return float(np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300))
