"""pytest configuration: the `gpu` marker and import paths.

`-m "not gpu"` runs everything that needs no GPU (oracle vs the reference's known answers, host
logic, C-ABI exports); `-m gpu` runs the parity tests of the CUDA path through the C ABI.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libparrygpu.so")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O
    return O


@pytest.fixture(scope="session")
def gpu_ctx():
    import parry_gb300 as pg
    from parry_gb300 import _build
    _build.build()
    ctx = pg.Context(device=0)
    yield ctx
    ctx.close()
