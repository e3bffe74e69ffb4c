import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "wgls-rs-fft_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG, ORACLE, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU; runs through the C ABI")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def lib_built():
    import gbfft
    return gbfft.build()


@pytest.fixture(scope="session")
def gpu_ctx(lib_built):
    import gbfft
    ctx = gbfft.Context(0)
    yield ctx
    ctx.close()


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))
