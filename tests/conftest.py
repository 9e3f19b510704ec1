"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libpbag kernels)")


@pytest.fixture(scope="session")
def lib():
    from pyblastafterglowmag_gb300 import build, _lib
    build.build()
    return _lib


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build_oracle()
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def reference():
    import pyoracle
    try:
        return pyoracle.Reference()
    except (FileNotFoundError, OSError) as e:
        pytest.skip(f"reference sources not available: {e}")


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return 0


def rel_l2_rows(x, y):
    """Per-row ||x - y||_2 / ||y||_2 over rows where y is not all zero, plus
    the number of rows where y is zero but x is not."""
    num = np.sqrt(((x - y) ** 2).sum(axis=1))
    den = np.sqrt((y ** 2).sum(axis=1))
    m = den > 0
    rel = num[m] / den[m] if m.any() else np.zeros(1)
    return rel, int(((den == 0) & (num > 0)).sum())
