import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "filament.jl_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

DECKS = os.path.join(ROOT, "tests", "decks")
PKG_DECKS = os.path.join(ROOT, "filament.jl_gb300", "decks")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
    config.addinivalue_line("markers", "slow: long CPU test")


@pytest.fixture(scope="session")
def oracle_binding():
    import oracle
    oracle.build()
    return oracle.binding()


@pytest.fixture(scope="session")
def gpu_lib():
    import build as b
    b.build()
    import filament_gb
    return filament_gb.load_library()
