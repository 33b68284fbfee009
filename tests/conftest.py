import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def golden_codes():
    return np.load(GOLDEN / "codes.npz")


@pytest.fixture(scope="session")
def kats():
    return np.load(GOLDEN / "kats.npz")


@pytest.fixture(scope="session")
def acq_golden():
    return np.load(GOLDEN / "acq_gps_l1_4mhz.npz")


def unpack_codes(fix, name):
    n = int(fix[name + "_len"])
    bits = np.unpackbits(fix[name], axis=1)[:, :n]
    return (1.0 - 2.0 * bits).astype(np.float32)


@pytest.fixture(scope="session")
def lib():
    from ugsdr_gb300 import _lib
    if not _lib.LIB_PATH.exists() and "UGSDR_CUDA_LIB" not in os.environ:
        # a fresh checkout: compile it (nvcc cross-compiles without a GPU)
        from ugsdr_gb300 import build
        build.build_library()
    return _lib.load()


@pytest.fixture(scope="session")
def ctx():
    from ugsdr_gb300.api import Context
    c = Context(int(os.environ.get("UGSDR_DEVICE", "0")))
    yield c
    c.close()


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.load()
    return pyoracle
