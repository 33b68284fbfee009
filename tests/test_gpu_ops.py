"""Per-op entry points (the Cuda* policies) against the reference's own
outputs (golden fixtures) and the oracle."""
import numpy as np
import pytest

from conftest import unpack_codes
from ugsdr_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def test_mix_bit_exact(ctx, kats):
    x = kats["mix_in"]
    for k, (fs, f, ph) in enumerate(kats["mix_params"]):
        y = x.copy()
        ctx.mix(y, fs, f, ph)
        np.testing.assert_array_equal(y, kats[f"mix_out_{k}"], err_msg=f"case {k}")


def test_mix_kat_half_rate(ctx, kats):
    y = np.ones(1000, np.complex64)
    ctx.mix(y, 1e6, 0.5e6)
    np.testing.assert_array_equal(y, kats["mix_half"])


@pytest.mark.parametrize("n", [1000, 4000, 2046, 511])
def test_dft(ctx, kats, n):
    v = kats[f"dft_in_{n}"]
    for inv, key in ((False, "fwd"), (True, "inv")):
        ref = kats[f"dft_{key}_{n}"]
        out = ctx.dft(v, inv)
        assert np.abs(out - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("n", [50000, 204600])
def test_dft_large_vs_oracle(ctx, oracle, n):
    rng = np.random.default_rng(n)
    v = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    lib = oracle.load()
    for inv in (0, 1):
        ref = np.empty(n, np.complex128)
        v64 = v.astype(np.complex128)
        lib.orc_dft_c2c_f64(v64.ctypes.data, ref.ctypes.data, n, inv)
        out = ctx.dft(v, bool(inv))
        assert np.abs(out - ref).max() <= 2e-5 * np.abs(ref).max()


def test_dft_beyond_four_step_columns(ctx):
    """2e7 points (400 ms at 50 MHz, the whole-signal DFT of the narrowband
    interference filter): past the size where four-column tiles fit, the
    split falls back to single columns.  numpy's FP64 FFT is the reference;
    the inverse carries the reference's 2/N scale."""
    n = 20_000_000
    rng = np.random.default_rng(20)
    v = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    ref = np.fft.fft(v.astype(np.complex128))
    out = ctx.dft(v)
    assert np.abs(out - ref).max() <= 2e-5 * np.abs(ref).max()
    back = ctx.dft(out, True)
    assert np.abs(back - 2 * v).max() <= 2e-5 * 2 * np.abs(v).max()


@pytest.mark.parametrize("name", ["glo", "ca4000"])
def test_matched_filter(ctx, kats, name):
    code = kats[f"mf_code_{name}"]
    spec = ctx.prepare_code_spectrum(code)
    ref_spec = kats[f"mf_spec_{name}"]
    assert np.abs(spec - ref_spec).max() <= 1e-5 * np.abs(ref_spec).max()
    out = ctx.filter_optimized(code.astype(np.complex64), spec)
    ref = kats[f"mf_out_{name}"]
    assert np.abs(out - ref).max() <= 1e-5 * np.abs(ref).max()
    if name == "glo":
        assert abs(out[0].real - 511) < 5e-3 and np.abs(out[1:].real + 1).max() < 5e-3


def test_abs_reshape_max_mean(ctx, kats):
    ab = ctx.abs(kats["abs_in"])
    np.testing.assert_allclose(ab, kats["abs_out"], rtol=2e-7)
    np.testing.assert_allclose(ctx.reshape_and_sum(kats["abs_out"], 1000), kats["reshape_out"], rtol=1e-6)
    with pytest.raises(L.UgsdrError):
        ctx.reshape_and_sum(kats["abs_out"], 3000)
    v, i = ctx.max_index(kats["abs_out"])
    assert i == int(kats["max_index"]) and v == float(kats["max_value"])
    m, s = ctx.mean_stddev(kats["abs_out"])
    assert abs(m - float(kats["mean"])) <= 1e-5 * abs(m) and abs(s - float(kats["sigma"])) <= 1e-4 * s
    assert ctx.mean_stddev(np.ones(1, np.float32)) == (0.0, 0.0)


def test_max_index_first_of_ties(ctx):
    x = np.zeros(100000, np.float32)
    x[[77, 5000, 99999]] = 3.0
    assert ctx.max_index(x) == (3.0, 77)


def test_correlate_kat(ctx, golden_codes):
    ca = unpack_codes(golden_codes, "gps_l1ca")[0]
    r = ctx.correlate(ca.astype(np.complex64), ca)
    assert r == complex(1023, 0)
    with pytest.raises(L.UgsdrError):
        ctx.correlate(ca.astype(np.complex64), ca[:-1])


def test_upsample_resample(ctx, kats, golden_codes):
    ca = unpack_codes(golden_codes, "gps_l1ca")
    np.testing.assert_array_equal(ctx.upsample(ca[3], 50000), kats["ups_ca3_50000"])
    x = kats["resample_in"]
    for k, (nf, of) in enumerate(kats["resample_pairs"]):
        ref = kats[f"resample_out_{k}"]
        out = ctx.resample(x, int(nf), int(of))
        assert out.shape == ref.shape
        np.testing.assert_array_equal(out, ref)  # the reference's float rounding, bit for bit


def test_convert_samples(ctx):
    raw8 = np.array([[-128, 127], [0, -1], [5, 7]], np.int8)
    np.testing.assert_array_equal(ctx.convert_samples(raw8, L.SAMPLES_CI8), np.array([-128 + 127j, -1j, 5 + 7j], np.complex64))
    raw16 = np.array([[-150, 16], [32767, -32768]], np.int16)  # iq_16_plus_16.bin first sample (-150, 16)
    np.testing.assert_array_equal(ctx.convert_samples(raw16, L.SAMPLES_CI16), np.array([-150 + 16j, 32767 - 32768j], np.complex64))
    real8 = np.array([-2, 3], np.int8)  # real_8.bin first sample -2
    np.testing.assert_array_equal(ctx.convert_samples(real8, L.SAMPLES_RI8), np.array([-2, 3], np.complex64))
