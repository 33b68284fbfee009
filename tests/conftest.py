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


# tracking-bank output rows (ugsdr_track_output) of the reference's own
# tracking history in tests/golden/track.npz: what the Observable pins feed
# to the oracle and to ugsdr_observables
TRACK_ROW = np.dtype([("taps", "<f4", (5, 2)), ("carrier_frequency", "<f8"), ("carrier_phase", "<f8"),
                      ("code_phase", "<f8"), ("code_frequency", "<f8"), ("phase_error", "<f8"), ("code_error", "<f8")])


def reference_track_rows(channels):
    """(n_epochs, len(channels)) rows from the reference tracker's outputs
    (make_golden.py track: E, P, L re/im, carrier_frequency, carrier_phase,
    code_phase, code_frequency, phase residual, code residual per epoch),
    plus each channel's starting carrier frequency."""
    z = np.load(GOLDEN / "track.npz")
    tr = [z[f"ch{k}/track"] for k in channels]
    rows = np.zeros((tr[0].shape[0], len(channels)), TRACK_ROW)
    for c, t in enumerate(tr):
        for tap, col in ((1, 0), (2, 2), (3, 4)):  # E, P, L in the VE/E/P/L/VL slots
            rows["taps"][:, c, tap, 0] = t[:, col]
            rows["taps"][:, c, tap, 1] = t[:, col + 1]
        for name, col in (("carrier_frequency", 6), ("carrier_phase", 7), ("code_phase", 8), ("code_frequency", 9),
                          ("phase_error", 10), ("code_error", 11)):
            rows[name][:, c] = t[:, col]
    return rows, [float(z[f"ch{k}/carrier_frequency"]) for k in channels], float(z["fs"])
