"""Shared test set-up: import paths, the `gpu` marker and golden fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "pd-flow_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (sm_103)")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def golden_qvga():
    return load_golden("qvga_s0.npz")


@pytest.fixture(scope="session")
def golden_vga():
    return load_golden("vga_s2.npz")


@pytest.fixture(scope="session")
def built_lib():
    """The CUDA library, built in tree if needed (nvcc cross-compiles on CPU)."""
    from pdflow import build
    build.build()
    from pdflow import _lib
    return _lib.load()
