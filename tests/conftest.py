import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def built():
    """Builds the in-tree libraries once per session (no-op when up to date)."""
    import __graft_entry__
    from hypercraft_gb300.build import build
    from oracle import bind
    build()
    bind.build_oracle()
    return __graft_entry__


@pytest.fixture(scope="session")
def oracle(built):
    from oracle import bind
    return bind.oracle()


@pytest.fixture(scope="session")
def reference(built):
    """The reference's own templates compiled here, or skip where its sources are absent."""
    from oracle import bind
    ref = bind.reference()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    return ref


@pytest.fixture(scope="session")
def ctx(built):
    from hypercraft_gb300 import mesher
    return mesher.Context(0)
