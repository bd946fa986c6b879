"""Test configuration: import paths, the `gpu` marker and shared fixtures.

`-m "not gpu"` tests run on any machine (oracle, host logic, C-ABI exports);
`-m gpu` tests need a CUDA device and call the library through its C ABI.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "webgpu-bcmc_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libbcmc_gb300.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def lib_built():
    import build as B

    return B.build()


@pytest.fixture(scope="session")
def ctx(lib_built):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bcmc

    return bcmc.Context(0)
