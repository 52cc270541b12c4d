import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "test-world_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def ptg():
    import ptgraph
    ptgraph.lib()
    return ptgraph


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def ctx(ptg):
    c = ptg.Ctx(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def ctx_grouped(ptg):
    """A context that stores every resident symmetric graph degree-grouped,
    however small (the default tuning groups graphs of 2^20+ edges)."""
    c = ptg.Ctx(0)
    c.set_tuning(vertex_order=2)
    yield c
    c.close()
