import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def reference_dir():
    """The reference source tree, present only in the build container."""
    d = os.environ.get("SM_REFERENCE_DIR", "/root/reference")
    return d if os.path.exists(os.path.join(d, "kdtree", "nanoflann.hpp")) else None


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle.pyoracle import lib
    return lib()
