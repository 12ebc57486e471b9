"""Shared fixtures; registers the ``gpu`` marker.

Tests marked ``gpu`` need a CUDA device and the built ``libmrsr.so``; the rest
run on the CPU (oracle pins, host logic, library loading and exports).
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device and the built libmrsr.so")


@pytest.fixture(scope="session")
def mr():
    import __graft_entry__ as ge
    return ge.package()


@pytest.fixture(scope="session")
def cuda(mr):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mr.library()
    return torch.device("cuda", 0)
