"""pytest configuration: the `gpu` marker, import paths and shared fixtures.

Tests marked `gpu` need a CUDA device (they call liblbmgpu.so through its C ABI and
compare against the CPU oracle).  Everything else runs on a CPU-only machine.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_ROOT = os.path.join(ROOT, "-2d-3d-_gb300")
for p in (ROOT, PKG_ROOT, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built liblbmgpu.so")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree if needed; skips nothing: a GPU test without it fails."""
    from lbmgpu import build as b
    b.build()
    import lbmgpu
    return lbmgpu.load_library()
