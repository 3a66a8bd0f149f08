import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def smoke_lib():
    """The in-tree CUDA library, built on demand (nvcc cross-compiles without a GPU)."""
    from smoke_simulation_gb300 import build
    build.build()
    import smoke_simulation_gb300 as smk
    return smk.lib()


@pytest.fixture(scope="session")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    from smoke_simulation_gb300 import build
    build.build()
    return torch.device("cuda:0")
