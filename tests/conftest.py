"""pytest configuration: the `gpu` marker and shared fixtures.

CPU-only tests (`-m "not gpu"`) exercise the oracle against the reference's golden
values, the host-side logic and the C-ABI library's exported symbols.  Tests marked
`gpu` need a GB300 and call the CUDA path through the C ABI.
"""
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the sm_103a kernels")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def pcg():
    """The product package with its native library built in-tree."""
    import physicore_gb300
    from physicore_gb300 import _build
    _build.build()
    physicore_gb300.load_library()
    return physicore_gb300
