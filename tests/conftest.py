"""Test configuration: the `gpu` marker and import paths.

`-m "not gpu"` runs on a CPU-only machine: the oracle against the golden
fixtures, the host tree and lists against the oracle, and the C-ABI library's
exports.  `-m gpu` runs the parity tests proper through the C ABI on a CUDA
device.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("hacc-coral_gb300", "oracle", "tests"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs through the C ABI)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle.Oracle()


@pytest.fixture(scope="session")
def hsr_lib():
    import build_ext
    build_ext.build()
    import hsr
    return hsr.load()


@pytest.fixture(scope="session")
def ctx(hsr_lib):
    import hsr
    c = hsr.Context(0)
    yield c
    c.close()
