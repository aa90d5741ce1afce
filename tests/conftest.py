"""Shared test configuration.

Markers: ``gpu`` -- needs a CUDA device (runs on the GPU host); everything else runs on CPU.
Every parity test compares the GPU path with the CPU oracle under oracle/.
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def repo_root():
    return REPO


@pytest.fixture(scope="session")
def data_root():
    import __graft_entry__ as ge
    return ge.data_root()


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN
