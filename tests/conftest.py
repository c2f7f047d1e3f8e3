import os
import sys
from pathlib import Path

# the oracle's LAPACK/BLAS calls run one BLAS thread each (also in the spawned
# workers of oracle.parallel); OpenBLAS reads this when it loads
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: long-running test")


@pytest.fixture(scope="session")
def pg():
    """The product package (pulsar.jl_gb300 imported as pulsar_gb300)."""
    import __graft_entry__ as ge
    ge._load_builder().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def ctx(pg):
    c = pg.Context(0)
    yield c
    c.close()
