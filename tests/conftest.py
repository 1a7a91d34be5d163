import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def fo():
    """The fluxoptics_gb300 package with its library loaded (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from __graft_entry__ import build, load_package
    build()
    pkg = load_package()
    pkg.load_library()
    return pkg


@pytest.fixture(scope="session")
def orc():
    from oracle import fluxoptics_oracle
    return fluxoptics_oracle
