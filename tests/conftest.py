import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def cuda_lib():
    """The CUDA library must load: GPU tests never fall back to anything else."""
    from deorbit_gb300 import build as B
    from deorbit_gb300 import sph

    if not os.path.exists(sph.LIB_PATH):
        B.build()
    return sph.lib()
