import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def gpu_ctx():
    import block_gb300

    ctx = block_gb300.Context(0)
    yield ctx
    ctx.close()


def conf(name):
    return os.path.join(GOLDEN, name, "dmrg.conf")
