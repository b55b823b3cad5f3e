"""Test configuration: markers and import paths.

`-m gpu` tests call the CUDA library through its C-ABI and compare with the
CPU oracle; everything else runs on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "opencfd-ec2d_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libec2d_gpu.so")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads libec2d_gpu.so; fails loudly without it."""
    import importlib
    b = importlib.import_module("ec2d_build")
    b.build()
    from ec2d import gpu
    gpu.lib()
    return gpu
