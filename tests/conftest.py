"""Shared test setup: import paths, the `gpu` marker, common fixtures."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "embree-aarch64_gb300")
for p in (PKG, os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


@pytest.fixture(scope="session")
def oracle():
    import oracle_ffi
    oracle_ffi.lib()
    return oracle_ffi


@pytest.fixture(scope="session")
def rtc():
    """The GPU library through its C ABI (GPU tests only)."""
    from rtcgb import api
    api.load()
    return api


@pytest.fixture(scope="session")
def device(rtc):
    d = rtc.Device(b"verbose=0")
    yield d
    d.release()
