import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libzgpu.so)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def zgpu():
    """The CUDA library, built in-tree if missing.  GPU tests only."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    from zombie_gb300 import build
    build.build()
    import zombie_gb300
    return zombie_gb300
