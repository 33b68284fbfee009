"""Interference stage on the device (STFT, JammingDetector,
JammingSuppressionEngine) against the reference's own outputs (golden
fixtures made through antijamming/jse.hpp) and the oracle.

Detections must match exactly in type, bin and frequency (J/N to 1e-4
relative: the peak / sigma of FP32 device magnitudes); samples are FP32
transforms of different association than the reference's FFT, compared with
an absolute tolerance of 1e-4 of the input's peak magnitude."""
from pathlib import Path

import numpy as np
import pytest

from ugsdr_gb300 import _lib as L

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / "golden" / "jamming.npz"
CASES = ("clean", "tone", "two_tones", "loud", "narrow", "narrow_4mhz")


def same_detections(got, ref, rel=1e-4):
    assert [d["type"] for d in got] == [r[0] for r in ref]
    assert [d["frequency_bin"] for d in got] == [r[1] for r in ref]
    assert [d["frequency"] for d in got] == [r[2] for r in ref]
    for d, r in zip(got, ref):
        assert abs(d["jammer_to_noise"] - r[3]) <= rel * abs(r[3])


def golden_detections(z, case):
    return list(zip(z[f"{case}_types"].tolist(), z[f"{case}_bins"].tolist(), z[f"{case}_freqs"].tolist(),
                    z[f"{case}_jn"].tolist()))


def test_stft_vs_reference(ctx):
    z = np.load(GOLDEN)
    cols = ctx.stft(z["tone_in"])
    ref = z["stft_cols"]
    assert cols.shape == ref.shape
    assert np.abs(cols - ref).max() <= 1e-5 * np.abs(ref).max()


def test_istft_vs_reference(ctx):
    z = np.load(GOLDEN)
    syn = ctx.istft(z["stft_cols"])
    ref = z["istft"]
    assert syn.shape == ref.shape
    assert np.abs(syn - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("case", CASES)
def test_suppress_vs_reference(ctx, case):
    z = np.load(GOLDEN)
    x = z[f"{case}_in"].copy()
    fs = float(z[f"{case}_fs"])
    det = ctx.jamming_suppress(x, fs)
    same_detections(det, golden_detections(z, case))
    ref = z[f"{case}_out"]
    assert np.abs(x - ref).max() <= 1e-4 * np.abs(z[f"{case}_in"]).max()
    if case == "clean":
        np.testing.assert_array_equal(x, z[f"{case}_in"])  # nothing detected: untouched


def test_detect_only(ctx):
    z = np.load(GOLDEN)
    for case in CASES:
        x = z[f"{case}_in"].copy()
        det = ctx.jamming_detect(x, float(z[f"{case}_fs"]))
        same_detections(det, golden_detections(z, case))
        np.testing.assert_array_equal(x, z[f"{case}_in"])


def test_device_pointer_matches_host(ctx):
    torch = pytest.importorskip("torch")
    z = np.load(GOLDEN)
    for case in ("tone", "narrow"):
        x = z[f"{case}_in"].copy()
        fs = float(z[f"{case}_fs"])
        host_det = ctx.jamming_suppress(x, fs)
        d = torch.from_numpy(z[f"{case}_in"].view(np.float32).copy()).cuda()
        ctx.set_stream(torch.cuda.current_stream().cuda_stream)
        try:
            dev_det = ctx.jamming_suppress(d.data_ptr(), fs, n=d.numel() // 2)
        finally:
            ctx.set_stream(None)
        torch.cuda.synchronize()
        assert dev_det == host_det
        np.testing.assert_array_equal(d.cpu().numpy().view(np.complex64), x)


def on_bin_tone(fs, n, k, amp):
    return amp * np.exp(2j * np.pi * (k * fs / 128) * np.arange(n) / fs)


@pytest.mark.parametrize("kind", ["wideband", "narrowband"])
def test_large_capture_vs_oracle(ctx, oracle, kind):
    """10 ms at 20 MHz (6247 STFT columns, a 200,000-point whole-signal DFT on
    the narrowband path).  Tones sit on STFT bin centres, so no magnitude is
    near the wideband threshold."""
    fs, n = 20e6, 200_000
    rng = np.random.default_rng(7 if kind == "wideband" else 8)
    x = rng.normal(0, 0.5, n) + 1j * rng.normal(0, 0.5, n)
    if kind == "wideband":
        x += on_bin_tone(fs, n, 20, 10.0)
    else:
        gate = (np.arange(n) // 128) % 20 == 0
        x += on_bin_tone(fs, n, 10, 10.0) + gate * on_bin_tone(fs, n, 50, 30.0)
    x = x.astype(np.complex64)
    ref_det, ref_y = oracle.jamming(x, fs)
    assert {d[0] for d in ref_det} == ({1, 2} if kind == "wideband" else {1})
    if kind == "wideband":
        mag = np.abs(oracle.stft(x))
        assert np.min(np.abs(mag - 20.0)) > 0.02
    y = x.copy()
    det = ctx.jamming_suppress(y, fs)
    same_detections(det, ref_det)
    assert np.abs(y - ref_y).max() <= 1e-4 * np.abs(x).max()


@pytest.mark.parametrize("window,overlap", [(100, 50), (256, 192), (64, 0)])
def test_stft_other_windows_vs_oracle(ctx, oracle, window, overlap):
    rng = np.random.default_rng(window)
    x = (rng.normal(size=5000) + 1j * rng.normal(size=5000)).astype(np.complex64)
    cols = ctx.stft(x, window, overlap)
    ref = oracle.stft(x, window, overlap)
    assert cols.shape == ref.shape
    assert np.abs(cols - ref).max() <= 1e-5 * np.abs(ref).max()
    syn = ctx.istft(ref, overlap)
    ref_syn = oracle.istft(ref, overlap)
    assert np.abs(syn - ref_syn).max() <= 1e-5 * np.abs(ref_syn).max()


def test_edges(ctx, oracle):
    # exactly one window: one column
    rng = np.random.default_rng(3)
    x = (rng.normal(0, 0.5, 128) + 1j * rng.normal(0, 0.5, 128) + on_bin_tone(2.048e6, 128, 9, 5.0)).astype(np.complex64)
    assert ctx.stft(x).shape == (1, 128)
    det, y = oracle.jamming(x, 2.048e6)
    got = ctx.jamming_suppress(x.copy(), 2.048e6)
    assert [(d["type"], d["frequency_bin"]) for d in got] == [(t, b) for t, b, _, _ in det]
    with pytest.raises(L.UgsdrError):
        ctx.stft(np.zeros(127, np.complex64))
    with pytest.raises(L.UgsdrError):
        ctx.jamming_suppress(np.zeros(100, np.complex64), 2.048e6)
    with pytest.raises(L.UgsdrError):
        ctx.stft(np.zeros(1000, np.complex64), 128, 128)


def test_mitigation_before_acquisition(ctx, oracle, golden_codes):
    """The front end's mitigation stage ahead of the search: Channel::
    GetSeveralEpochs suppresses (dfe/dfe.hpp:199-202) the samples that
    FastSearchEngineBase::Process then searches (acquisition/fse.hpp:456-460).
    A CW jammer 55 dB above the noise hides three GPS L1 C/A satellites; the
    device suppresses it in place and the batched search runs on the same
    device buffer.  Peaks (code phase, Doppler bin) equal the oracle chain's
    (oracle engine, then oracle acquisition), levels within 1e-4 of its FP64
    search."""
    torch = pytest.importorskip("torch")
    from conftest import unpack_codes
    from ugsdr_gb300 import signals
    ca = unpack_codes(golden_codes, "gps_l1ca")
    fs, n, k = 4e6, 4000, 10
    sats = [(3, 100.5, 1500.0), (11, 700.25, -2500.0), (17, 333.0, 500.0)]
    ems = [signals.Emitter(ca[p], 1.023e6, cp, dop, 50.0, data_rate=0.0) for p, cp, dop in sats]
    x = signals.synthesize(ems, fs, n * k, 0.5, "cf32", seed=21)
    # on STFT bin 40 (1.25 MHz at 4 MHz): no magnitude near the wideband threshold
    x = (x + 400 * np.exp(2j * np.pi * 1.25e6 * np.arange(n * k) / fs)).astype(np.complex64)
    assert np.min(np.abs(np.abs(oracle.stft(x)) - 20.0)) > 0.02
    det_ref, y_ref = oracle.jamming(x, fs)
    assert det_ref and {d[0] for d in det_ref} == {1, 2}

    def search(samples, on_device):
        hs = [ctx.code_put(ca[p], n) for p, _, _ in sats]
        try:
            job = ctx.make_job(samples, L.SAMPLES_CF32, fs, n, k, hs, 5000, 500, n_samples=n * k, on_device=on_device)
            return ctx.acquire(job)
        finally:
            for h in hs:
                ctx.code_release(h)

    # jammed: the satellites are not found at their true code phase
    blind = search(x, False)
    assert any(r.snr < 2.0 for r in blind)
    d = torch.from_numpy(x.view(np.float32).copy()).cuda()
    torch.cuda.synchronize()
    det = ctx.jamming_suppress(d.data_ptr(), fs, n=n * k)
    same_detections(det, det_ref)
    res = search(d.data_ptr(), True)
    for (p, cp, dop), r in zip(sats, res):
        code = oracle.upsample(ca[p], n)
        o32 = oracle.acquire(y_ref, n, k, code, fs, 5000, 500)
        o64 = oracle.acquire(y_ref, n, k, code, fs, 5000, 500, double=True)
        assert r.index == int(o32["index"]) and r.doppler_bin == int(o32["doppler_bin"]), (p, r, o32)
        assert abs(r.index - cp * fs / 1.023e6) <= 1 and r.doppler == pytest.approx(dop)
        assert abs(r.level - o64["level"]) <= 1e-4 * o64["level"]
        assert r.snr > 3.3
