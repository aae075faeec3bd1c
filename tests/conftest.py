import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests")


@pytest.fixture(scope="session")
def built():
    """Builds libvrtx and the oracle once per session."""
    import __graft_entry__ as g

    g.build()
    return True


@pytest.fixture()
def device(built):
    from visrtx_gb300 import anari

    dev = anari.Device(0)
    if not dev.is_valid():
        pytest.fail("libvrtx found no CUDA device: " + "; ".join(dev.errors()))
    yield dev
    dev.release()
