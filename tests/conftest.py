import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine's kernels)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import binding

    binding.build()
    return binding.lib()


@pytest.fixture(scope="session")
def engine():
    """Build (if needed) and load the CUDA engine; GPU tests only."""
    from rrtl_gb300 import build, sim

    build.build()
    sim.lib()
    return sim


@pytest.fixture(scope="session")
def ctx(engine):
    return engine.default_context()
