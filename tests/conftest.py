"""Test configuration: the `gpu` marker, import paths, and on-demand builds of the oracle and of
libsemgb (both compile on machines without a GPU)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "proxy-geos-hc_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libsemgb kernels)")


@pytest.fixture(scope="session")
def semgb_lib():
    import build as semgb_build  # proxy-geos-hc_gb300/build.py
    semgb_build.build()
    import semgb
    return semgb


@pytest.fixture(scope="session")
def cuda_device():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return 0
