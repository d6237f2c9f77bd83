import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); calls the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def built():
    """Build the in-tree libraries once per session (no-op when up to date)."""
    from oracle import build as oracle_build
    from orion_gb300 import build
    return {"product": build.build_product(), "sobol": build.sobol_table(), **oracle_build.build_all()}


@pytest.fixture(scope="session")
def ctx(built):
    import orion_gb300 as og
    c = og.Context(0)
    yield c
    c.close()
