import os
import sys

import pytest

# Every tree created by the tests checks its whole device structure (links,
# per-child counts and AABBs) after each mutation.
os.environ.setdefault("IKDG_DEBUG_VALIDATE", "1")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("ikd-tree_gb300", "oracle"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libikdg kernels)")


@pytest.fixture(scope="session")
def ikdg_mod():
    import ikdg
    ikdg.load()
    return ikdg


@pytest.fixture(scope="session")
def cpu_kinds():
    """CPU implementations to compare against: the unmodified reference when
    its library was built (oracle/_ref, from the reference install), and the
    oracle port, which always builds."""
    import oracle_lib
    if not oracle_lib.available("port"):
        oracle_lib.build("port")
    return (["ref"] if oracle_lib.available("ref") else []) + ["port"]
