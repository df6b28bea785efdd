"""Shared pytest configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and the built libmlpgpu.so; everything
else runs on the CPU (oracle, golden fixtures, host logic, C-ABI exports).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "wamca-gpu-mi_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and libmlpgpu.so")


@pytest.fixture(scope="session")
def mlpgpu_mod():
    import mlpgpu

    if mlpgpu.device_count() < 1:
        pytest.fail("no CUDA device visible to a test marked gpu")
    return mlpgpu
