"""Shared test set-up: the gpu marker, the in-tree build and the repository root on sys.path."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from dpgsolver_gb300 import _build

    _build.build_all()
    yield
