"""Test configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a GB300 and the built librn_ao.so; everything else runs on a CPU
host. The oracle (oracle/) is what the GPU results are compared against.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "raw-native_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 (sm_103) and the built librn_ao.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build(with_ref=False) if not os.path.exists(O.LIB) else None
    return O


@pytest.fixture(scope="session")
def rn():
    """The GPU library; a gpu test that cannot load it fails (there is no fallback)."""
    import rn_ao
    rn_ao.init()
    return rn_ao
