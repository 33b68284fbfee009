"""Packed front-end captures (BBP DDC, NT1065) decoded on the device: the
per-op unpack is bit-exact with the reference's own readers, the tracking
bank and the acquisition front end take packed input directly, and a search
of the reference's real BBP DDC capture (GPS L1, 33.25 MHz, 1-bit I/Q)
matches the oracle chain decode -> resample -> ProcessBpsk."""
from pathlib import Path

import numpy as np
import pytest

from conftest import unpack_codes
from test_gpu_acquire import RTOL, check_vs_oracle
from ugsdr_gb300 import _lib as L

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden" / "packed.npz"


def golden():
    z = np.load(GOLD)
    g = z["bbp_decoded"].astype(np.float32)
    return z, (g[:, 0] + 1j * g[:, 1]).astype(np.complex64)


def test_unpack_bit_exact(ctx):
    z, bbp = golden()
    fs = float(z["bbp_fs"])
    np.testing.assert_array_equal(ctx.unpack_samples(z["bbp_raw"], L.SAMPLES_BBP_DDC, fs), bbp)
    nt = np.arange(256, dtype=np.uint8)
    for ch in range(4):
        g = z[f"nt1065_{ch}"].astype(np.float32)
        out = ctx.unpack_samples(nt, L.SAMPLES_NT1065_1 + ch, 50e6)
        np.testing.assert_array_equal(out, (g[:, 0] + 1j * g[:, 1]).astype(np.complex64))


def test_real_bbp_capture_acquisition(ctx, oracle, golden_codes):
    """10 ms of the real capture: BBP DDC bytes in, decoded and resampled
    33.25 -> 6.65 MHz (the rate the reference's AdjustSamplingRate picks for
    33.25 MHz, fse.hpp:222-240) by the job's front end, 1 ms blocks x 10,
    +-5 kHz at 200 Hz (the reference's integration-test grid)."""
    z, bbp = golden()
    ca = unpack_codes(golden_codes, "gps_l1ca")
    prns = [8, 22, 2, 6]  # PRN 9 and 23 are above the 3.3 threshold in this slice
    handles = [ctx.code_put(ca[p], 6650) for p in prns]
    try:
        job = ctx.make_job(z["bbp_raw"], L.SAMPLES_BBP_DDC, 6.65e6, 6650, 10, handles, 5000.0, 200.0,
                           input_sampling_rate=33.25e6, code_offset_ratio=5.0)
        res = ctx.acquire(job)
    finally:
        for h in handles:
            ctx.code_release(h)
    y = oracle.resample(bbp, 6650000, 33250000)
    for p, r in zip(prns, res):
        code = oracle.upsample(ca[p], 6650)
        kw = dict(ratio=5.0)
        check_vs_oracle(r, oracle.acquire(y, 6650, 10, code, 6.65e6, 5000, 200, **kw),
                        oracle.acquire(y, 6650, 10, code, 6.65e6, 5000, 200, double=True, **kw))
    assert res[0].snr > 3.3 and res[1].snr > 3.3


def test_packed_track_and_nt1065_front_end(ctx, golden_codes):
    """Tracking takes BBP DDC bytes (decoded on the device first) with the same
    taps as decoded complex input; an NT1065 acquisition job equals the same
    job on the decoded real samples."""
    from ugsdr_gb300.api import TrackBank
    z, bbp = golden()
    ca = unpack_codes(golden_codes, "gps_l1ca")
    chans = [dict(code=0, fs=33.25e6, code_frequency=1.023e6, code_phase=15145.0, carrier_frequency=-600.0)]
    a = TrackBank(ctx, chans, [ca[8]])
    b = TrackBank(ctx, chans, [ca[8]])
    out_packed = a.run(z["bbp_raw"], L.SAMPLES_BBP_DDC, 10)
    out_cf = b.run(bbp, L.SAMPLES_CF32, 10)
    a.close()
    b.close()
    np.testing.assert_array_equal(out_packed["taps"], out_cf["taps"])
    np.testing.assert_array_equal(out_packed["code_phase"], out_cf["code_phase"])
    rng = np.random.default_rng(3)
    nt = rng.integers(0, 256, 4000 * 4, dtype=np.uint8)
    h = ctx.code_put(ca[3], 4000)
    try:
        for ch in range(4):
            dec = ctx.unpack_samples(nt, L.SAMPLES_NT1065_1 + ch, 4e6)
            r1 = ctx.acquire(ctx.make_job(nt, L.SAMPLES_NT1065_1 + ch, 4e6, 4000, 4, [h], 2000.0, 500.0))
            r2 = ctx.acquire(ctx.make_job(dec, L.SAMPLES_CF32, 4e6, 4000, 4, [h], 2000.0, 500.0))
            assert (r1[0].index, r1[0].doppler_bin) == (r2[0].index, r2[0].doppler_bin)
            assert abs(r1[0].level - r2[0].level) <= RTOL * r2[0].level
    finally:
        ctx.code_release(h)
