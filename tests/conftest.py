"""Test configuration.

Markers: `gpu` marks tests that need a CUDA device (run with `-m gpu` on a GB300); the
rest run on CPU (`-m "not gpu"`). The oracle (oracle/liborc.so) is built on demand.
"""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libgfgpu.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(os.path.join(GOLDEN, name)))
    return load


@pytest.fixture(scope="session")
def gpulib():
    """libgfgpu.so built for this machine and loaded (GPU tests only)."""
    from galaxy_formation_gb300 import _lib, build

    build.build()
    lib = _lib.load()
    assert lib.nbody_num_threads() > 0, "no usable CUDA device"
    return lib


def rel_err(a, b):
    """Per-particle relative error |a - b| / |b| of (n, 3) arrays."""
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)
