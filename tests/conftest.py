import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def rrlib():
    """librr.so, built from csrc/ if it is missing or stale."""
    from radeonrays_sdk_gb300 import build, rr
    build.build()
    return rr.lib()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ctx(rrlib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from radeonrays_sdk_gb300 import rr
    c = rr.Context()
    yield c
    c.close()


def golden(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


MESH_FIXTURES = ["soup256", "height17", "one", "two", "three", "dupes", "planar", "u16"]
