"""Shared pytest configuration: the ``gpu`` marker and import paths."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("", "oracle", "polyfields.jl_gb300", "tests/golden"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpolyfields_gpu.so")


GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture
def golden_dir():
    return GOLDEN
