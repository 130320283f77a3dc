"""Shared test setup.

Markers: `gpu` for tests that need a GB300 (they call the CUDA library
through its C-ABI). Everything else runs on the CPU: the oracle against
the golden vectors, host-side logic, and the library's exported symbols.
"""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the library's kernels)")


@pytest.fixture(scope="session", autouse=True)
def _built_oracle():
    """The oracle is test infrastructure: build it once if it is missing."""
    from oracle import build as ob
    if not os.path.exists(ob.LIB):
        ob.build_oracle()
    yield


@pytest.fixture(scope="session")
def built_library():
    """libhairsim.so, built in tree if missing (nvcc cross-compiles on CPU)."""
    from barbu_gb300 import build as bb
    if not os.path.exists(bb.LIB):
        bb.build()
    return bb.LIB
