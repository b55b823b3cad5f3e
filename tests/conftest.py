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

# The reference's own input files (control.in, bc2d_1.in, Mesh2d.dat of its
# RAE2822 case) are read from EC2D_REFERENCE_DIR, by default the read-only
# reference checkout of the build container.  Tests that need them skip, with
# the reason in the summary (pytest -rs), where the directory is absent.
REFERENCE_DIR = os.environ.get("EC2D_REFERENCE_DIR", "/root/reference")


def reference_file(name):
    """Path of one of the reference's input files, or a skip naming why."""
    path = os.path.join(REFERENCE_DIR, name)
    if not os.path.exists(path):
        pytest.skip(f"reference input {name} not found under EC2D_REFERENCE_DIR={REFERENCE_DIR}")
    return path


def pytest_report_header(config):
    have = os.path.exists(os.path.join(REFERENCE_DIR, "Mesh2d.dat"))
    return f"reference inputs (EC2D_REFERENCE_DIR): {REFERENCE_DIR} ({'found' if have else 'absent: those tests skip'})"


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
