"""Pins the CPU oracle (oracle/oracle.cpp) against the reference's own
primitives: every golden vector in tests/golden/ was produced by the
reference sources compiled into oracle/_ref (tests/golden/make_golden.py)."""
import numpy as np
from pathlib import Path
import pytest

from conftest import GOLDEN, unpack_codes


def test_table_mixer_bit_exact(oracle, kats):
    x = kats["mix_in"]
    for k, (fs, f, ph) in enumerate(kats["mix_params"]):
        np.testing.assert_array_equal(oracle.table_mix(x, fs, f, ph), kats[f"mix_out_{k}"], err_msg=f"case {k}")
        y64 = oracle.table_mix(x.astype(np.complex128), fs, f, ph)
        np.testing.assert_array_equal(y64, kats[f"mix_out64_{k}"], err_msg=f"case {k} f64")


def test_mixer_kat_half_rate(oracle, kats):
    y = oracle.table_mix(np.ones(1000, np.complex64), 1e6, 0.5e6)
    np.testing.assert_array_equal(y, kats["mix_half"])
    # basic_tests.cpp:321-357: alternating +-1, imag ~ 0
    np.testing.assert_array_equal(y.real, 1.0 - 2.0 * (np.arange(1000) & 1))
    assert np.abs(y.imag).max() < 1e-6


@pytest.mark.parametrize("n", [1000, 4000, 2046, 511])
def test_dft(oracle, kats, n):
    lib = oracle.load()
    v = kats[f"dft_in_{n}"]
    for inv, key in ((0, "fwd"), (1, "inv")):
        out = np.empty_like(v)
        lib.orc_dft_c2c_f32(v.ctypes.data, out.ctypes.data, n, inv)
        ref = kats[f"dft_{key}_{n}"]
        assert np.abs(out - ref).max() <= 1e-6 * np.abs(ref).max() + 1e-6


def test_dft_tone_kat(oracle):
    # basic_tests.cpp:482-505: 1000-point tone at 0.1 fs peaks at bin 100 with value N
    lib = oracle.load()
    n = 1000
    x = np.exp(2j * np.pi * 0.1 * np.arange(n)).astype(np.complex64)
    out = np.empty_like(x)
    lib.orc_dft_c2c_f32(x.ctypes.data, out.ctypes.data, n, 0)
    assert np.argmax(np.abs(out)) == 100
    assert abs(abs(out[100]) - n) < 5e-3 * n


@pytest.mark.parametrize("name", ["glo", "ca4000"])
def test_matched_filter(oracle, kats, name):
    lib = oracle.load()
    code = kats[f"mf_code_{name}"]
    spec = np.empty(code.size, np.complex64)
    lib.orc_prepare_code_spectrum_f32(code.ctypes.data, code.size, 0, spec.ctypes.data)
    ref_spec = kats[f"mf_spec_{name}"]
    assert np.abs(spec - ref_spec).max() <= 1e-6 * np.abs(ref_spec).max()
    sig = code.astype(np.complex64)
    lib.orc_filter_optimized_f32(sig.ctypes.data, sig.size, spec.ctypes.data, 0)
    ref = kats[f"mf_out_{name}"]
    assert np.abs(sig - ref).max() <= 1e-5 * np.abs(ref).max()
    if name == "glo":
        # basic_tests.cpp:368-383
        assert abs(sig[0].real - 511) < 5e-3
        assert np.abs(sig[1:].real + 1).max() < 5e-3


def test_reductions(oracle, kats):
    lib = oracle.load()
    a = kats["abs_in"]
    ab = np.empty(a.size, np.float32)
    lib.orc_abs_f32(a.ctypes.data, a.size, ab.ctypes.data)
    np.testing.assert_allclose(ab, kats["abs_out"], rtol=2e-7)
    r = kats["abs_out"].copy()
    assert lib.orc_reshape_sum_f32(r.ctypes.data, r.size, 1000) == 0
    np.testing.assert_array_equal(r[:1000], kats["reshape_out"])
    assert lib.orc_reshape_sum_f32(r.ctypes.data, 10000, 3000) == -1
    ab_ref = kats["abs_out"]
    assert lib.orc_max_index_f32(ab_ref.ctypes.data, 10000) == int(kats["max_index"])
    m, s = np.zeros(1, np.float32), np.zeros(1, np.float32)
    lib.orc_mean_std_f32(ab_ref.ctypes.data, 10000, m.ctypes.data, s.ctypes.data)
    assert m[0] == kats["mean"] and s[0] == kats["sigma"]


def test_correlator_kat(oracle, kats, golden_codes):
    ca = unpack_codes(golden_codes, "gps_l1ca")[0]
    out = np.zeros(2, np.float32)
    sig = ca.astype(np.complex64)
    oracle.load().orc_correlate_f32(sig.ctypes.data, ca.ctypes.data, 1023, out.ctypes.data)
    assert out[0] == 1023 and out[1] == 0  # basic_tests.cpp:72-86
    assert complex(*out) == complex(kats["correlate_ca"][0])


def test_upsampler(oracle, kats, golden_codes):
    ca = unpack_codes(golden_codes, "gps_l1ca")
    np.testing.assert_array_equal(oracle.upsample(ca[3], 50000), kats["ups_ca3_50000"])


def test_resampler(oracle, kats):
    x = kats["resample_in"]
    for k, (nf, of) in enumerate(kats["resample_pairs"]):
        out = oracle.resample(x, int(nf), int(of))
        ref = kats[f"resample_out_{k}"]
        assert out.shape == ref.shape
        np.testing.assert_array_equal(out, ref)  # same sequential float sum


def test_acquisition_matches_reference(oracle, acq_golden, golden_codes):
    ca = unpack_codes(golden_codes, "gps_l1ca")
    iq = acq_golden["acq_raw"].astype(np.float32)
    x = (iq[:, 0] + 1j * iq[:, 1]).astype(np.complex64)
    for prn, rec, rec64 in zip(acq_golden["acq_prns"], acq_golden["acq_rec"], acq_golden["acq_rec64"]):
        code = oracle.upsample(ca[prn], 4000)
        r = oracle.acquire(x, 4000, 10, code, 4e6, 5000, 500)
        # index and Doppler bin bit-exact against the reference's float path
        assert r["index"] == rec[4] and r["doppler_bin"] == rec[5], prn
        assert abs(r["level"] - rec[0]) <= 1e-4 * rec[0]
        r64 = oracle.acquire(x, 4000, 10, code, 4e6, 5000, 500, double=True)
        assert r64["index"] == rec64[4] and r64["doppler_bin"] == rec64[5]
        assert abs(r64["level"] - rec64[0]) <= 1e-9 * rec64[0]
        assert abs(r64["snr"] - rec64[6]) <= 1e-9 * rec64[6]


def test_packed_decoders(oracle):
    """The oracle's BBP DDC / NT1065 decoders against the reference's own
    readers (SignalParametersBase::GetSeveralMs on the real BBP capture,
    NtlabPackedSpan on every byte value)."""
    z = np.load(Path(__file__).parent / "golden" / "packed.npz")
    g = z["bbp_decoded"].astype(np.float32)
    np.testing.assert_array_equal(oracle.unpack_bbp(z["bbp_raw"], float(z["bbp_fs"])), g[:, 0] + 1j * g[:, 1])
    assert oracle.bbp_epoch_bytes(float(z["bbp_fs"])) == int(z["bbp_epoch_bytes"])
    for ch in range(4):
        g = z[f"nt1065_{ch}"].astype(np.float32)
        np.testing.assert_array_equal(oracle.unpack_nt1065(np.arange(256, dtype=np.uint8), ch), g[:, 0] + 1j * g[:, 1])


JAMMING_CASES = ("clean", "tone", "two_tones", "loud", "narrow", "narrow_4mhz")


@pytest.mark.parametrize("case", JAMMING_CASES)
def test_jamming_engine(oracle, case):
    """The oracle's JammingSuppressionEngine::Process against the reference's
    own (antijamming/jse.hpp through the reference harness): detections and
    suppressed samples bit for bit, for the clean, wideband (tone, two
    tones, loud) and narrowband (gated second tone) paths."""
    z = np.load(Path(__file__).parent / "golden" / "jamming.npz")
    det, y = oracle.jamming(z[f"{case}_in"], float(z[f"{case}_fs"]))
    assert [d[0] for d in det] == list(z[f"{case}_types"])
    assert [d[1] for d in det] == list(z[f"{case}_bins"])
    assert [d[2] for d in det] == list(z[f"{case}_freqs"])
    assert [d[3] for d in det] == list(z[f"{case}_jn"])
    np.testing.assert_array_equal(y, z[f"{case}_out"])
    det_only, y_in = oracle.jamming(z[f"{case}_in"], float(z[f"{case}_fs"]), suppress=False)
    assert det_only == det
    np.testing.assert_array_equal(y_in, z[f"{case}_in"])


def test_stft_round_trip(oracle):
    """ShortTimeFourierTransform split and OverlapAndAdd (math/stft.hpp) against
    the reference's, bit for bit; the periodic Hann window at 75 % overlap
    sums to 2 and the inverse is scaled 2 / 128, so the interior of the
    synthesis is 4 x the input."""
    z = np.load(Path(__file__).parent / "golden" / "jamming.npz")
    cols = oracle.stft(z["tone_in"])
    np.testing.assert_array_equal(cols, z["stft_cols"])
    syn = oracle.istft(cols)
    np.testing.assert_array_equal(syn, z["istft"])
    x = z["tone_in"]
    np.testing.assert_allclose(syn[96:len(syn) - 96], 4 * x[96:len(syn) - 96], rtol=0, atol=1e-4 * np.abs(x).max())


PREAMBLE_CASES = ("gps_two_subframes", "gps_inverted", "gps_odd_length", "gps_shorter_than_preamble", "gps_zeros",
                  "glonass_strings", "glonass_odd_length", "glonass_shorter_than_preamble")


@pytest.mark.parametrize("case", PREAMBLE_CASES)
def test_preamble_search(oracle, case):
    """FindPreambleGps / Glonass's candidate epochs: the oracle's FP64 matched
    filter against the reference's own float one (SequentialMatchedFilter +
    SequentialAbs over sign(prompt I), thresholds 153 / 370), and both
    against the exact integer correlation they approximate (|y| = 2 |sum of
    +-1 products|, so every value is a multiple of 4 away from a threshold
    that is not)."""
    z = np.load(Path(__file__).parent / "golden" / "preamble.npz")
    x = z[f"{case}/prompt_i"].astype(np.float32)
    msg = int(z[f"{case}/message"])
    got = oracle.preamble_search(x, msg, cap=len(x))
    assert got == z[f"{case}/indexes"].tolist()
    sym = [1, -1, -1, -1, 1, -1, 1, 1] if msg == 0 else None
    if sym is not None:
        b = np.where(x > 0, 1, -1)
        p = np.repeat(sym, 20)[: len(x)]
        s = np.array([int(np.dot(np.roll(b, -k)[: len(p)], p)) for k in range(len(x))])
        assert np.flatnonzero(2 * np.abs(s) > 153).tolist() == got


def test_observables_oracle(oracle):
    """Observable's arithmetic (observable.hpp:75-88) on a synthetic history:
    sigma equals the reference's SequentialMeanStdDev, the SNR follows
    27 + 20 log10(|I| / sigma) in float, the pseudorange offset is the
    truncated ms of the preamble epoch, and the phase the reference's radian
    accumulation."""
    z = np.load(Path(__file__).parent / "golden" / "preamble.npz")
    q = z["sigma/prompt_q"]
    n = len(q)
    rng = np.random.default_rng(5)
    rows = np.zeros(n, [("taps", "<f4", (5, 2)), ("carrier_frequency", "<f8"), ("phase_error", "<f8"),
                        ("code_phase", "<f8")])
    rows["taps"][:, 2, 0] = rng.normal(0, 300, n).astype(np.float32)
    rows["taps"][:, 2, 1] = q
    rows["carrier_frequency"] = 1500.0 + np.cumsum(rng.normal(0, 0.01, n))
    rows["phase_error"] = rng.normal(0, 0.02, n)
    rows["code_phase"] = 2345.678 - np.arange(n) * 1e-3
    fs, if_hz, f0, ph0, pos, corr = 4e6, 1000.0, 1499.5, 0.3, 17, 68.0
    o = oracle.observables(rows, fs, if_hz, f0, ph0, pos, corr)
    sigma = z["sigma/value"]
    snr = np.float32(27) + np.float32(20) * np.log10(np.abs(rows["taps"][:, 2, 0]) / sigma)
    np.testing.assert_allclose(o[:, 3], snr, rtol=0, atol=1e-5)  # dB: a float ulp near 27
    s2ms = 1000 / fs
    off = int(rows["code_phase"][pos] * s2ms)
    np.testing.assert_array_equal(o[:, 0], rows["code_phase"] * s2ms - off + corr)
    np.testing.assert_array_equal(o[:, 2], rows["carrier_frequency"] - if_hz)
    f_prev = np.concatenate([[f0], rows["carrier_frequency"][:-1]])
    cycles = ph0 / (2 * np.pi) + np.cumsum(f_prev / 1000 + rows["phase_error"] / 4)
    np.testing.assert_allclose(o[:, 1], -cycles + np.arange(1, n + 1) * if_hz / 1e3, rtol=0, atol=1e-8)


# ---------------------------------------------------------------- tracking
def _track_fixture():
    z = np.load(GOLDEN / "track.npz")
    raw = z["samples"].astype(np.float32)
    x = (raw[:, 0] + 1j * raw[:, 1]).astype(np.complex64)
    fix = np.load(GOLDEN / "codes.npz")
    chips = {0: unpack_codes(fix, "gps_l1ca"), 6: unpack_codes(fix, "galileo_e1b")}
    chans = []
    for k in range(int(z["channels"])):
        pre = f"ch{k}/"
        chans.append(dict(signal=int(z[pre + "signal"]), chips=chips[int(z[pre + "signal"])][int(z[pre + "prn"])],
                          base=float(z[pre + "code_frequency"]), code_phase=float(z[pre + "code_phase"]),
                          carrier_frequency=float(z[pre + "carrier_frequency"]), track=z[pre + "track"],
                          refine_code_phase=float(z[pre + "refine_code_phase"]), refine=z[pre + "refine"]))
    return float(z["fs"]), x, chans


def test_track_taps_pinned_to_reference(oracle):
    """The oracle's per-epoch taps (track_oracle.cpp, the reference NCO mode)
    from the reference tracker's own state at each epoch equal the
    reference's E / P / L (CorrelateSplit with TableMixer wipe-off,
    tracking_parameters.hpp:472-493, tracker.hpp:119-139) to 1e-5 of the
    epoch's prompt: the reference sums in float, the oracle in double."""
    fs, x, chans = _track_fixture()
    spm = int(fs / 1000)
    for ch in chans:
        tr = ch["track"]
        period_ms = int(round(len(ch["chips"]) / ch["base"] * 1000))
        for e in range(tr.shape[0]):
            cf, cph, cp = (ch["carrier_frequency"], 0.0, ch["code_phase"]) if e == 0 else (tr[e - 1, 6], tr[e - 1, 7], tr[e - 1, 8])
            ph = cp - fs / 1e3 * (e % period_ms)
            o = oracle.track_taps(x[e * spm:(e + 1) * spm], ch["chips"], fs, ch["base"], ph, cf, cph, 0.25, 0.25, nco_mode=1)
            mine = np.array([o[2] + 1j * o[3], o[4] + 1j * o[5], o[6] + 1j * o[7]])
            ref = tr[e, 0:6:2] + 1j * tr[e, 1:6:2]
            assert np.abs(mine - ref).max() <= 1e-5 * abs(ref[1]), (ch["signal"], e, mine, ref)


def test_track_loop_pinned_to_reference(oracle):
    """The oracle's loop update (Pll then Dll in the reference's types and
    order, UpdatePhase before the taps) fed the reference's taps reproduces
    the reference's state after every epoch (tracking_parameters.hpp:163-165,
    495-528): carrier frequency, carrier phase, code phase, code frequency."""
    fs, _, chans = _track_fixture()
    for ch in chans:
        tr = ch["track"]
        loop = oracle.track_loop(tr[:, :6], fs, ch["base"], ch["code_phase"], ch["carrier_frequency"])
        for col_loop, col_ref in ((0, 6), (1, 7), (2, 8), (3, 9), (4, 10), (5, 11)):
            np.testing.assert_allclose(loop[:, col_loop], tr[:, col_ref], rtol=1e-12, atol=1e-12)


def test_track_refine_pinned_to_reference(oracle):
    """AddSignalImpl's refinement restated (pyoracle.track_refine) gives the
    reference's offset, acceptance and refined code phase on every channel
    (GPS L1 C/A 1 ms codes and a Galileo E1B 4 ms code)."""
    fs, x, chans = _track_fixture()
    channels = [dict(fs=fs, code=i, code_frequency=ch["base"], code_phase=ch["refine_code_phase"],
                     carrier_frequency=ch["carrier_frequency"]) for i, ch in enumerate(chans)]
    acc, offs, phases, _ = oracle.track_refine(x, channels, [ch["chips"] for ch in chans])
    for i, ch in enumerate(chans):
        assert offs[i] == int(ch["refine"][0]) and acc[i] == int(ch["refine"][1]) and phases[i] == ch["refine"][2], i


def test_observables_pinned_to_reference(oracle):
    """The oracle's Observable arithmetic (orc_observables_f64) on the
    reference tracker's own histories gives the reference Observable's
    outputs (tests/golden/observables.npz: constructor, CalculateSnr,
    UpdateScale + UpdatePseudoranges; IF 1.25 kHz, preamble at epoch 37,
    time of week 345678 s): pseudorange, pseudophase and Doppler bit for
    bit, SNR within 1e-12."""
    from conftest import reference_track_rows
    z = np.load(GOLDEN / "observables.npz")
    rows, cf0, fs = reference_track_rows(range(int(z["channels"])))
    if_hz, pos = float(z["intermediate_frequency"]), int(z["position"])
    # UpdatePseudorangeGps after UpdateScale: time_scale[i] - (i - pos + tow_ms + 2) = 70 - 2
    for c in range(rows.shape[1]):
        got = oracle.observables(rows[:, c], fs, if_hz, cf0[c], 0.0, pos, 68.0)
        ref = z[f"ch{c}"]
        np.testing.assert_array_equal(got[:, 0], ref[:, 0])
        np.testing.assert_array_equal(got[:, 1], ref[:, 1])
        np.testing.assert_array_equal(got[:, 2], ref[:, 2])
        np.testing.assert_allclose(got[:, 3], ref[:, 3], rtol=1e-12, atol=0)
