"""Test configuration: the `gpu` marker and import paths.

`-m "not gpu"` runs on any host (oracle, host logic, C-ABI symbol checks);
`-m gpu` needs a CUDA device and calls the CUDA path through the C-ABI.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "gpu-isac_gb300"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpulib():
    """The CUDA library, built if needed; GPU tests fail (not skip) without it."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("gpuisac_build", os.path.join(ROOT, "gpu-isac_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    from gpuisac import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch.device("cuda:0")
