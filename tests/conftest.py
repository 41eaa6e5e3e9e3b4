"""Shared test configuration.

`-m gpu` tests run the CUDA engine through its C ABI; everything else runs
on the CPU (oracle port against the reference's golden fixtures, host
compiler, library symbol table).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "ngspice-sf-mirror_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def golden(name: str):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


@pytest.fixture(scope="session")
def built_lib():
    """The product library, built in-tree (nvcc cross-compiles without a GPU)."""
    from ngspice_gb300 import build
    return build.build()
