import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# the warp_cfd sources, read by CPU tests that check fixtures against them when present
REFERENCE = os.environ.get("WCFD_REFERENCE", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libwcfd.so")


@pytest.fixture(scope="session")
def built_lib():
    from warpcfd_gb300.build import build_library

    return build_library()
