import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "wavelet-suffix-fm-index_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the kernels)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build(ref=False)
    return O


@pytest.fixture(scope="session")
def wtg():
    import wtg as W
    W.build()
    return W
