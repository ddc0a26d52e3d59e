"""Shared test setup: the `gpu` marker, repository import path, and helpers.

`-m "not gpu"` runs on a host without a GPU: the oracle against the golden
fixtures, the host logic and the C ABI surface of libgpujoin.so.  `-m gpu`
runs the parity tests proper: the CUDA kernels through the C ABI against
the CPU oracle.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity tests of the sm_103a kernels)")


@pytest.fixture(scope="session")
def orc():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)
    import oracle

    return oracle


@pytest.fixture(scope="session")
def gj():
    import gpujoin_gb300

    gpujoin_gb300.lib()
    return gpujoin_gb300


@pytest.fixture(scope="session")
def cuda(gj):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda:0")
