import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgpu4snn.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import g4s_oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def g4s():
    import gpu4snn_gb300
    from gpu4snn_gb300 import build
    build.build()
    gpu4snn_gb300.load()
    return gpu4snn_gb300
