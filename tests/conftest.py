import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libfmmbem.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle_py

    oracle_py.lib()
    return oracle_py


@pytest.fixture(scope="session")
def fm():
    """The product package; GPU tests fail loudly if the CUDA library is not built."""
    import fmbem_gpu_c_gb300 as fm

    fm.lib()
    return fm
