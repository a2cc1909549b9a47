import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The voting stage folds every accumulator into a fingerprint (statistics column 4) only when
# asked; the tests compare it with the oracle's, so the whole session asks.
os.environ.setdefault("SM_VOTE_FINGERPRINT", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def reference_dir():
    """The reference source tree (present only where the reference's sources are), as the
    oracle's build recipe for the reference probes locates it; None when absent."""
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_probe"))
    try:
        import build_ref
    finally:
        sys.path.pop(0)
    return build_ref.REF if build_ref.available() else None


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle.pyoracle import lib
    return lib()
