import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "cpp-pt_gb300"))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def golden():
    def get(name):
        return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))
    return get


@pytest.fixture(scope="session")
def gpu_lib():
    """The in-tree CUDA library; a GPU test fails (not skips) when it is absent."""
    from cpppt import lib
    import torch
    assert torch.cuda.is_available(), "GPU test without a CUDA device"
    return lib.load()
