"""Shared fixtures: the package (loaded by path), the CPU oracle, and the `gpu` marker.

Tests marked `gpu` run the CUDA library on a GB300; the rest run on any CPU and never touch
the device (the library is loaded there only to check its exported symbols)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and liblbm_gb300.so")


@pytest.fixture(scope="session")
def lbm():
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def O():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def lbm_gpu(lbm):
    """The package with liblbm_gb300.so built for sm_103a and loaded; skips without a GPU."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lbm.build()
    lbm._native.lib()
    return lbm
