"""C-ABI checks that need no GPU: the library loads, exports every symbol the
header declares, and its host-side code generation matches the reference's
own generators (golden fixtures from tests/golden/make_golden.py)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT, unpack_codes
from ugsdr_gb300 import _lib as L
from ugsdr_gb300 import api


def header_functions():
    text = (ROOT / "include" / "ugsdr_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(ugsdr_[a-z_0-9]+)\s*\(", text, flags=re.M)))


def test_exports_every_header_symbol(lib):
    names = header_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(L.SIGNATURES), set(names) ^ set(L.SIGNATURES)


def test_abi_version(lib):
    assert lib.ugsdr_abi_version() == 9  # four-step tile shapes (warp-owned rows) and the autotuner


@pytest.mark.parametrize("name,signal,count", [("gps_l1ca", L.GPS_L1CA, 37), ("gps_l5i", L.GPS_L5I, 32),
                                               ("gps_l5q", L.GPS_L5Q, 32), ("glonass_l1of", L.GLONASS_L1OF, 1),
                                               ("galileo_e1b", L.GALILEO_E1B, 50), ("galileo_e1c", L.GALILEO_E1C, 50)])
def test_prn_codes_bit_exact(golden_codes, name, signal, count):
    ref = unpack_codes(golden_codes, name)
    assert ref.shape[0] == count
    for sv in range(count):
        np.testing.assert_array_equal(api.prn_code(signal, sv), ref[sv], err_msg=f"{name} sv {sv}")


def test_prn_code_errors(lib):
    buf = np.empty(2000, np.float32)
    n = C.c_size_t()
    # GPS C/A has 37 ids (GpsL1Ca.hpp:22-23 throws beyond)
    assert lib.ugsdr_prn_code(L.GPS_L1CA, 37, buf.ctypes.data, buf.size, C.byref(n)) == L.E_INVALID
    assert lib.ugsdr_prn_code(L.GPS_L5I, 32, buf.ctypes.data, buf.size, C.byref(n)) == L.E_INVALID
    assert lib.ugsdr_prn_code(L.GALILEO_E1B, 50, buf.ctypes.data, buf.size, C.byref(n)) == L.E_INVALID
    assert lib.ugsdr_prn_code(L.GALILEO_E1C, 0, buf.ctypes.data, buf.size, C.byref(n)) == L.E_INVALID
    assert n.value == 8184
    assert lib.ugsdr_prn_code(L.GPS_L2CM, 0, buf.ctypes.data, buf.size, C.byref(n)) == L.E_UNSUPPORTED
    # too small a buffer reports the length
    assert lib.ugsdr_prn_code(L.GPS_L1CA, 0, buf.ctypes.data, 10, C.byref(n)) == L.E_INVALID
    assert n.value == 1023


def test_repeat_upsample_matches_reference(kats, golden_codes):
    ca = unpack_codes(golden_codes, "gps_l1ca")
    e1b = unpack_codes(golden_codes, "galileo_e1b")
    np.testing.assert_array_equal(api.repeat_upsample(ca[3], 1, 50000), kats["ups_ca3_50000"])
    np.testing.assert_array_equal(api.repeat_upsample(e1b[0], 1, 200000), kats["ups_e1b0_200000"])
    np.testing.assert_array_equal(api.repeat_upsample(ca[5], 4, 16000), kats["ups_ca5_rep4_16000"])


def test_doppler_grid_counts():
    assert api.doppler_bins(5000, 500) == 21
    assert api.doppler_bins(5000, 250) == 41
    assert api.doppler_bins(5000, 62.5) == 161
    assert api.doppler_bins(5000, 25) == 401
    assert api.doppler_bins(0, 100) == 1
    with pytest.raises(L.UgsdrError):
        api.doppler_bins(5000, 0)


def test_galileo_codes_are_boc(golden_codes):
    for name in ("galileo_e1b", "galileo_e1c"):
        c = unpack_codes(golden_codes, name)
        assert c.shape == (50, 8184)
        np.testing.assert_array_equal(c[:, 0::2], -c[:, 1::2])  # DecodeBoc [c, -c]


def test_capture_sizes(lib):
    """ugsdr_sample_bytes: BBP DDC epochs as SignalParametersBase::OpenFile sizes
    them (33.25 MHz: 16,640 bytes per 1 ms), one byte per NT1065 sample."""
    import ctypes as C
    b = C.c_size_t()
    assert lib.ugsdr_sample_bytes(4, 33.25e6, 33250 * 10, C.byref(b)) == 0 and b.value == 166400
    assert lib.ugsdr_sample_bytes(5, 50e6, 1000, C.byref(b)) == 0 and b.value == 1000
    assert lib.ugsdr_sample_bytes(2, 4e6, 1000, C.byref(b)) == 0 and b.value == 4000
    assert lib.ugsdr_sample_bytes(4, 33.25e6, 33250 + 1, C.byref(b)) != 0  # not whole epochs
    assert lib.ugsdr_sample_bytes(4, 33.2505e6, 33250, C.byref(b)) != 0    # not a whole-kHz rate
