"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # build libtc / the oracle in-tree if a fresh checkout has not built them yet
    from trianglecount_gb300 import build as B
    if not os.path.exists(B.LIBTC):
        B.build_libtc()
    B.build_oracle()


@pytest.fixture(scope="session")
def ctx():
    import trianglecount_gb300 as tc
    c = tc.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(ROOT, "tests", "golden")
