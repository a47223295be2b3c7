import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def golden_host():
    import numpy as np
    return np.load(os.path.join(GOLDEN, "ref_host.npz"))


@pytest.fixture(scope="session")
def golden_gpu():
    import numpy as np
    path = os.path.join(GOLDEN, "ref_kernels.npz")
    if not os.path.exists(path):
        pytest.skip("tests/golden/ref_kernels.npz not generated yet")
    return np.load(path)
