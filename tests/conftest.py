"""Shared test configuration.

``-m gpu`` tests need a CUDA device and the built library; the rest run on
CPU (oracle against golden vectors, host logic, C-ABI exports).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libgbsym.so")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle.orc()


@pytest.fixture(scope="session")
def ref():
    import oracle
    r = oracle.ref()
    if r is None:
        pytest.skip("reference source tree not available here")
    return r


@pytest.fixture(scope="session")
def gpu():
    """Built library + CUDA device; fails loudly when either is missing."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test collected without a CUDA device")
    from sympiler_gb300 import _lib
    _lib.lib()
    torch.cuda.init()
    return torch.device("cuda:0")
