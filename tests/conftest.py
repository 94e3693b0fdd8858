import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    from oracle.bind import Oracle, build
    build()
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "ref_vectors.npz"))


@pytest.fixture(scope="session")
def gpu():
    """The built library on a CUDA device; fails loudly if either is missing."""
    import torch
    from mtgp_gb300 import build as b
    b.build()
    from mtgp_gb300._lib import lib
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    torch.cuda.init()
    return lib()
