import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_ROOT = os.path.join(ROOT, "slim-release-apps_gb300")
for p in (ROOT, PKG_ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    # keep the collection order stable: files in alphabetical order, tests in file order
    return None


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from h3d import build

    build.build()
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def golden_small():
    import numpy as np

    return dict(np.load(os.path.join(GOLDEN, "stencil_small.npz")))


@pytest.fixture(scope="session")
def golden_band():
    """Band-storage goldens from the compiled Hmvp_MT_mex / sweep_MT_mex (make_golden.py)."""
    import numpy as np

    return dict(np.load(os.path.join(GOLDEN, "band_small.npz")))
