import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import bsam_oracle
    bsam_oracle.lib()
    return bsam_oracle


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as ge
    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def ctx(pkg):
    c = pkg.Context(0)
    yield c
    c.close()
