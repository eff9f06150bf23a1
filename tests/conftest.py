import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """Build the libraries (no-op when up to date)."""
    import __graft_entry__ as g

    g.build()
    return True


@pytest.fixture(scope="session")
def oracle(built):
    from oracle.oracle import Oracle

    return Oracle()


@pytest.fixture(scope="session")
def ctx_exact(built):
    from phoebus_gb300.fluid import FluidContext

    c = FluidContext(0, exact=True)
    yield c
    c.close()


@pytest.fixture(scope="session")
def ctx_fast(built):
    from phoebus_gb300.fluid import FluidContext

    c = FluidContext(0, exact=False)
    yield c
    c.close()
