"""Shared test setup: the `gpu` marker, import paths, and an in-tree build of
libsdpg.so (nvcc cross-compiles without a GPU, so CPU tests load it too)."""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def sdpg():
    build = importlib.import_module("sdpa-gmp_gb300.build")
    build.build()
    return importlib.import_module("sdpa-gmp_gb300")


@pytest.fixture(scope="session")
def exact():
    return importlib.import_module("oracle.exact")


@pytest.fixture(scope="session")
def problems():
    return importlib.import_module("sdpa-gmp_gb300.problems")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
