import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if stale) and loads the CUDA library; the GPU tests need it."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from olcao_gb300 import build, api
    build.build()
    return api.lib()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "primitives.npz"))


@pytest.fixture(scope="session")
def gpu_free_lib():
    """Builds (if stale) and loads the library for its host-only entry points
    (argument checks, dataset writers); needs no GPU."""
    from olcao_gb300 import build, api
    build.build()
    return api.lib()
