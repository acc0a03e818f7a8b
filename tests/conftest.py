import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cuda-pro-cell_gb300")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: long-running (large workloads)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def built():
    """Build libprocell.so and the CLI (cross-compiles without a GPU)."""
    sys.path.insert(0, PKG)
    import build as pkg_build
    pkg_build.build()
    return pkg_build


@pytest.fixture(scope="session")
def engine(built, oracle_lib):
    from procell import Engine
    eng = Engine(0)
    yield eng
    eng.close()
