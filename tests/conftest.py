import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built engine library")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as entry

    return entry.package()


@pytest.fixture(scope="session")
def O():
    from oracle import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def engine_lib(pkg):
    sys.path.insert(0, os.path.join(ROOT, "cfd-craft_gb300"))
    try:
        import build as b
    finally:
        sys.path.pop(0)
    b.build()
    return pkg.engine.load()
