import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.join(ROOT, "tests")
GOLDEN = os.path.join(TESTS, "golden")
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def shaw():
    """The product library (built in-tree if needed)."""
    import shaw_gb300
    shaw_gb300.build()
    return shaw_gb300


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (test infrastructure)."""
    import oracle_lib
    oracle_lib.build()
    return oracle_lib


def mesh_dir(name):
    return os.path.join(GOLDEN, "meshes", name)
