"""pytest configuration: the `gpu` marker and shared fixtures.

Tests marked gpu need a GB300 (they run the CUDA path through the C ABI);
everything else runs on the CPU: the oracle against golden vectors, the
host-side logic of the product library, and the C-ABI surface.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and runs the CUDA path")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def ctx():
    import whir_gb300 as W
    c = W.Context(0)
    yield c
    c.close()
