"""Test configuration: the `gpu` marker and shared fixtures.

`-m "not gpu"` runs the oracle known-answer tests, the host logic and the
C-ABI export check (no GPU needed); `-m gpu` runs the parity tests of the
CUDA path against the oracle and the golden fixtures.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def vf():
    """The product package with its CUDA library built (GPU tests only)."""
    from voxelfragmentml_gb300 import build as B
    B.build()
    import voxelfragmentml_gb300 as V
    V.lib()
    return V


@pytest.fixture(scope="session")
def ctx(vf):
    c = vf.Context(0)
    yield c
    c.close()
