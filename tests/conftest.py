import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "vcl-volume-scanner_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds (if stale) the product libraries and the oracle."""
    import vs_build
    import build_oracle

    vs_build.build()
    build_oracle.build_oracle()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    import vs_scanner

    if vs_scanner.device_count() < 1:
        pytest.fail("no CUDA device visible to libvs_gb300.so")
    return True
