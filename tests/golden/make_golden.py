"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own CPU primitives, compiled from the reference sources
by `make -C oracle ref REF_DIR=...` into oracle/_ref/libugsdr_ref.so
(oracle/ref_harness.cpp + project FFTW-API shim), and stores their outputs as
small .npz fixtures.  Only this script needs the reference tree; the tests
read the committed fixtures.

    python tests/golden/make_golden.py [REF_DIR [FIXTURE ...]]
"""
from __future__ import annotations

import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from ugsdr_gb300 import signals  # noqa: E402

SIGNALS = {  # ugsdr::Signal value -> (name, count of ids)
    0: ("gps_l1ca", 37),
    2: ("gps_l5i", 32),
    3: ("gps_l5q", 32),
    4: ("glonass_l1of", 1),
    6: ("galileo_e1b", 50),
    7: ("galileo_e1c", 50),
}


def ref_lib(ref_dir: str) -> C.CDLL:
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref", f"REF_DIR={ref_dir}"], check=True)
    lib = C.CDLL(str(ROOT / "oracle" / "_ref" / "libugsdr_ref.so"))
    vp, sz, d, i = C.c_void_p, C.c_size_t, C.c_double, C.c_int
    lib.ref_prn_code.argtypes = [i, i, vp, i]
    lib.ref_repeat_upsample.argtypes = [vp, i, i, vp, sz]
    lib.ref_table_mixer_f32.argtypes = [vp, sz, d, d, d]
    lib.ref_table_mixer_f64.argtypes = [vp, sz, d, d, d]
    lib.ref_dft_c2c_f32.argtypes = [vp, vp, sz, i]
    lib.ref_dft_r2c_f32.argtypes = [vp, vp, sz]
    lib.ref_prepare_code_spectrum_f32.argtypes = [vp, sz, vp]
    lib.ref_filter_optimized_f32.argtypes = [vp, sz, vp]
    lib.ref_abs_f32.argtypes = [vp, sz, vp]
    lib.ref_reshape_sum_f32.argtypes = [vp, sz, sz, vp]
    lib.ref_reshape_sum_f32.restype = i
    lib.ref_max_index_f32.argtypes = [vp, sz, vp, vp]
    lib.ref_mean_std_f32.argtypes = [vp, sz, vp, vp]
    lib.ref_resample_c32.argtypes = [vp, sz, vp, sz, sz, sz]
    lib.ref_resample_c32.restype = sz
    lib.ref_correlate_f32.argtypes = [vp, vp, sz, vp]
    lib.ref_acquire_f32.argtypes = [vp, sz, sz, sz, vp, d, d, d, d, d, i, i, vp, vp]
    lib.ref_acquire_f64.argtypes = [vp, sz, sz, sz, vp, d, d, d, d, d, i, i, vp, vp]
    lib.ref_bbp_read.argtypes = [C.c_char_p, d, d, sz, vp]
    lib.ref_bbp_read.restype = C.c_long
    lib.ref_nt1065_decode.argtypes = [vp, sz, i, vp]
    lib.ref_preamble_filter_f32.argtypes = [vp, sz, i, vp]
    lib.ref_stft_f32.argtypes = [vp, sz, vp, sz]
    lib.ref_stft_f32.restype = C.c_long
    lib.ref_istft_f32.argtypes = [vp, sz, vp]
    lib.ref_jamming_process_f32.argtypes = [vp, sz, d, vp, vp, vp, vp, i]
    lib.ref_jamming_process_f32.restype = i
    return lib


def p(a: np.ndarray) -> int:
    return a.ctypes.data


def codes(lib) -> dict[str, np.ndarray]:
    out = {}
    buf = np.zeros(20000, np.float32)
    for sig, (name, count) in SIGNALS.items():
        rows = []
        for sv in range(count):
            n = lib.ref_prn_code(sig, sv, p(buf), buf.size)
            rows.append(buf[:n].copy())
        arr = np.stack(rows)
        assert set(np.unique(arr)) <= {-1.0, 1.0}
        out[name] = np.packbits(arr < 0, axis=1)
        out[name + "_len"] = np.array(arr.shape[1])
    return out


def unpack(fix, name: str) -> np.ndarray:
    n = int(fix[name + "_len"])
    bits = np.unpackbits(fix[name], axis=1)[:, :n]
    return (1.0 - 2.0 * bits).astype(np.float32)


def kats(lib, code_fix) -> dict[str, np.ndarray]:
    rng = np.random.default_rng(7)
    out = {}
    ca = unpack(code_fix, "gps_l1ca")
    glo = unpack(code_fix, "glonass_l1of")[0]
    # mixer: several (fs, f, phase), float and double, n = 3000
    x = (rng.normal(size=3000) + 1j * rng.normal(size=3000)).astype(np.complex64)
    out["mix_in"] = x
    mixes = [(4e6, 1234.5, 0.0), (4e6, -4500.0, 0.0), (4e6, 1.5e6, 1.0), (1e6, 0.5e6, 0.0), (50e6, -14.58e6, -2.5),
             (4e6, 0.0, 0.3)]
    out["mix_params"] = np.array(mixes)
    for k, (fs, f, ph) in enumerate(mixes):
        y = x.copy()
        lib.ref_table_mixer_f32(p(y), y.size, fs, f, ph)
        out[f"mix_out_{k}"] = y
        y64 = x.astype(np.complex128)
        lib.ref_table_mixer_f64(p(y64), y64.size, fs, f, ph)
        out[f"mix_out64_{k}"] = y64
    # ones mixed at fs/2 (basic_tests.cpp:321-357)
    ones = np.ones(1000, np.complex64)
    lib.ref_table_mixer_f32(p(ones), ones.size, 1e6, 0.5e6, 0.0)
    out["mix_half"] = ones
    # DFT KAT tone (basic_tests.cpp:482-505) and random c2c both directions
    for n in (1000, 4000, 2046, 511):
        v = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
        fwd = np.empty_like(v)
        inv = np.empty_like(v)
        lib.ref_dft_c2c_f32(p(v), p(fwd), n, 0)
        lib.ref_dft_c2c_f32(p(v), p(inv), n, 1)
        out[f"dft_in_{n}"] = v
        out[f"dft_fwd_{n}"] = fwd
        out[f"dft_inv_{n}"] = inv
    # code spectra and matched filter: GLONASS KAT (basic_tests.cpp:368-383), C/A at 4000 samples
    for name, code in (("glo", glo), ("ca4000", None)):
        if code is None:
            code = np.empty(4000, np.float32)
            lib.ref_repeat_upsample(p(ca[0]), 1023, 1, p(code), 4000)
        code = np.ascontiguousarray(code, np.float32)
        spec = np.empty(code.size, np.complex64)
        lib.ref_prepare_code_spectrum_f32(p(code), code.size, p(spec))
        sig = code.astype(np.complex64)
        lib.ref_filter_optimized_f32(p(sig), sig.size, p(spec))
        out[f"mf_code_{name}"] = code
        out[f"mf_spec_{name}"] = spec
        out[f"mf_out_{name}"] = sig
    # abs / reshape / max / mean-std / correlator
    a = (rng.normal(size=10000) + 1j * rng.normal(size=10000)).astype(np.complex64)
    ab = np.empty(a.size, np.float32)
    lib.ref_abs_f32(p(a), a.size, p(ab))
    out["abs_in"], out["abs_out"] = a, ab
    rs = np.empty(1000, np.float32)
    assert lib.ref_reshape_sum_f32(p(ab), ab.size, 1000, p(rs)) == 0
    out["reshape_out"] = rs
    assert lib.ref_reshape_sum_f32(p(ab), ab.size, 3000, p(rs)) != 0  # 10000 % 3000 != 0 throws
    mv, mi = C.c_float(), C.c_size_t()
    lib.ref_max_index_f32(p(ab), ab.size, C.byref(mv), C.byref(mi))
    out["max_value"], out["max_index"] = np.array(mv.value, np.float32), np.array(mi.value)
    m, s = C.c_float(), C.c_float()
    lib.ref_mean_std_f32(p(ab), ab.size, C.byref(m), C.byref(s))
    out["mean"], out["sigma"] = np.array(m.value, np.float32), np.array(s.value, np.float32)
    sig = ca[0].astype(np.complex64)
    cor = np.empty(1, np.complex64)
    lib.ref_correlate_f32(p(sig), p(ca[0]), 1023, p(cor))
    out["correlate_ca"] = cor
    # upsampler ramp (basic_tests.cpp:764-850) and code upsampling
    up = np.empty(50000, np.float32)
    lib.ref_repeat_upsample(p(ca[3]), 1023, 1, p(up), 50000)
    out["ups_ca3_50000"] = up
    e1b = unpack(code_fix, "galileo_e1b")[0]
    up2 = np.empty(200000, np.float32)
    lib.ref_repeat_upsample(p(e1b), e1b.size, 1, p(up2), 200000)
    out["ups_e1b0_200000"] = up2
    up3 = np.empty(16000, np.float32)
    lib.ref_repeat_upsample(p(ca[5]), 1023, 4, p(up3), 16000)
    out["ups_ca5_rep4_16000"] = up3
    # resampler: complex ramp 1000 samples at several rate pairs
    ramp = (np.arange(1000) + 1j * np.arange(1000)[::-1]).astype(np.complex64)
    out["resample_in"] = ramp
    pairs = [(2, 3), (3, 2), (1023, 2000), (4, 4)]
    out["resample_pairs"] = np.array(pairs)
    for k, (nf, of) in enumerate(pairs):
        n_out = lib.ref_resample_c32(p(ramp), ramp.size, None, 0, nf, of)
        dst = np.empty(n_out, np.complex64)
        lib.ref_resample_c32(p(ramp), ramp.size, p(dst), n_out, nf, of)
        out[f"resample_out_{k}"] = dst
    return out


def acquisition(lib, code_fix) -> dict[str, np.ndarray]:
    """Full-size GPS L1 C/A acquisition (int8 IQ, 4 MHz, 10 ms, 1 ms x 10 blocks,
    +-5 kHz / 500 Hz) on a seeded synthetic capture, reference primitives in
    float and double, for 8 PRNs (the 6 visible + 2 absent)."""
    ca = unpack(code_fix, "gps_l1ca")
    codes = {i: ca[i] for i in range(32)}
    raw, truth = signals.gps_l1_config(seed=1, codes=codes)
    iq = raw.astype(np.float32).reshape(-1)  # int8 -> float exactly (GetPartialSignal)
    visible = [t["prn"] for t in truth]
    absent = [p_ for p_ in range(32) if p_ not in visible][:2]
    prns = visible + absent
    recs, recs64, outs = [], [], []
    fs, n, k = 4.0e6, 4000, 10
    for prn in prns:
        code = np.empty(n, np.float32)
        lib.ref_repeat_upsample(p(ca[prn]), 1023, 1, p(code), n)
        rec = np.zeros(7)
        best = np.zeros(n, np.float32)
        lib.ref_acquire_f32(p(iq), iq.size // 2, n, k, p(code), fs, 5000.0, 500.0, 0.0, 1.0, 0, 1, p(rec), p(best))
        recs.append(rec)
        outs.append(best)
        iq64 = iq.astype(np.float64)
        code64 = code.astype(np.float64)
        rec64 = np.zeros(7)
        lib.ref_acquire_f64(p(iq64), iq64.size // 2, n, k, p(code64), fs, 5000.0, 500.0, 0.0, 1.0, 0, 1, p(rec64), None)
        recs64.append(rec64)
    return dict(acq_raw=raw, acq_prns=np.array(prns), acq_visible=np.array(visible), acq_rec=np.array(recs),
                acq_rec64=np.array(recs64), acq_best=np.array(outs),
                acq_truth=np.array([[t["prn"], t["doppler"], t["code_phase_samples"], t["cn0"]] for t in truth]))


def bbp_epoch_bytes(fs: float) -> int:
    """Bytes per 1 ms BbpDdc epoch (signal_parameters.hpp:78-85): 4 bits per
    complex sample in 64-bit words plus a header word, padded to an even count."""
    words = fs / 1e3 * 4 / 64 + 1
    b = int(words / 2) * 2
    if words % 2:
        b += 2
    return b * 8


def packed(lib, ref_dir: str) -> dict[str, np.ndarray]:
    """Packed front-end formats: the first 10 ms of the reference's real
    BbpDdc capture (GPS L1, 33.25 MHz; fs and centre frequency as in
    benchmark/benchmark.cpp:82) decoded by the reference's own reader, and
    every NT1065 byte value decoded for each of the four channels."""
    out = {}
    path = Path(ref_dir) / "data" / "bbp_ddc_gps_L1.dat"
    fs, ms = 33.25e6, 10
    eb = bbp_epoch_bytes(fs)
    raw = np.fromfile(path, np.uint8, count=eb * ms)
    dec = np.zeros(int(fs / 1e3) * ms * 2, np.float32)
    n = lib.ref_bbp_read(str(path).encode(), 1575.42e6, fs, ms, p(dec))
    assert n == int(fs / 1e3) * ms
    out["bbp_raw"] = raw
    out["bbp_fs"] = np.array(fs)
    out["bbp_epoch_bytes"] = np.array(eb)
    out["bbp_decoded"] = dec.reshape(-1, 2).astype(np.int8)  # values are +-1
    nt = np.arange(256, dtype=np.uint8)
    for ch in range(4):
        d = np.zeros(512, np.float32)
        lib.ref_nt1065_decode(p(nt), nt.size, ch, p(d))
        out[f"nt1065_{ch}"] = d.reshape(-1, 2).astype(np.int8)  # values -3, -1, 1, 3 (imag 0)
    return out


# real_8 acquisition known answer (test/integration_tests.cpp:253-263, the
# reference's expected GPS L1 C/A results for its real_8.bin capture: sv id,
# Doppler Hz, code offset in 38.192 MHz samples; a run passes when >= 4 of
# them are found within 400 Hz, 237-241)
REAL8_KAT = [(2, 0, 34213), (5, 6000, 28203), (8, -1000, 4695), (14, 0, 36321), (17, 2000, 20725),
             (20, 3000, 13404), (21, 0, 6289), (25, 5000, 26828)]


def real8(ref_dir: str) -> dict[str, np.ndarray]:
    """The first 4 ms (FastSearchEngineBase's ms_to_process) of the
    reference's real_8.bin: real int8 at 38.192 MHz, centre 1575.42 MHz +
    9.55 MHz (integration_tests.cpp:76), with the known answer."""
    fs = 38.192e6
    raw = np.fromfile(Path(ref_dir) / "data" / "real_8.bin", np.int8, count=int(fs / 1e3) * 4)
    assert raw[0] == -2  # integration_tests.cpp:124-141
    return {"samples": raw, "fs": np.array(fs), "if_hz": np.array(9.55e6),
            "kat": np.array(REAL8_KAT, np.float64)}


def iq16(ref_dir: str) -> dict[str, np.ndarray]:
    """The first 4 ms of the reference's iq_16_plus_16.bin (int16 I/Q at 4 MHz,
    centre on L1; integration_tests.cpp:75), whose acquisition test asks a
    non-empty result (401-404)."""
    raw = np.fromfile(Path(ref_dir) / "data" / "iq_16_plus_16.bin", np.int16, count=16000 * 2).reshape(-1, 2)
    assert tuple(raw[0]) == (-150, 16)  # integration_tests.cpp:105-122
    return {"samples": raw, "fs": np.array(4e6)}


JAMMING_CASES = {  # name -> (fs, n, seed); signals built by jamming_input()
    "clean": (2.048e6, 2048, 11),
    "tone": (2.048e6, 2048, 12),
    "two_tones": (2.048e6, 2048, 13),
    "loud": (2.048e6, 2048, 14),
    "narrow": (2.048e6, 2048, 15),
    "narrow_4mhz": (4e6, 4000, 16),
}


def jamming_input(name: str, fs: float, n: int, seed: int) -> np.ndarray:
    """Noise (sigma 0.5 per part) plus the case's interferers: CW tones, a
    loud one over loud noise, and for the narrowband cases a weak steady tone
    with a stronger tone gated on in one 128-sample slot of twenty."""
    rng = np.random.default_rng(seed)
    t = np.arange(n) / fs
    x = rng.normal(0, 0.5, n) + 1j * rng.normal(0, 0.5, n)
    if name == "tone":
        x += 10 * np.exp(2j * np.pi * 0.5e6 * t)
    elif name == "two_tones":
        x += 10 * np.exp(2j * np.pi * 0.5e6 * t) + 5 * np.exp(2j * np.pi * -0.7e6 * t)
    elif name == "loud":
        x = 40 * x + 200 * np.exp(2j * np.pi * 0.3e6 * t)
    elif name.startswith("narrow"):
        gate = (np.arange(n) // 128) % 20 == 0
        x += 10 * np.exp(2j * np.pi * 0.25e6 * t) + gate * 30 * np.exp(2j * np.pi * 0.9e6 * t)
    return x.astype(np.complex64)


def jamming(lib) -> dict[str, np.ndarray]:
    """JammingSuppressionEngine<complex<float>>::Process (in place) on seeded
    signals through the reference's own code, plus its STFT (128 / 96) and
    OverlapAndAdd on the tone case.  In the cases the wideband filter runs
    on, every STFT magnitude stays at least 0.1 % away from its threshold 20,
    so an FP32 device transform takes the same zeroing decisions."""
    out = {}
    for name, (fs, n, seed) in JAMMING_CASES.items():
        x = jamming_input(name, fs, n, seed)
        iq = np.ascontiguousarray(x).view(np.float32).copy()
        types = np.zeros(64, np.int32)
        bins = np.zeros(64, np.int64)
        freqs = np.zeros(64)
        jn = np.zeros(64)
        cnt = lib.ref_jamming_process_f32(p(iq), n, fs, p(types), p(bins), p(freqs), p(jn), 64)
        cols = lib.ref_stft_f32(p(np.ascontiguousarray(x).view(np.float32)), n, None, 0)
        spec = np.zeros(cols * 128 * 2, np.float32)
        lib.ref_stft_f32(p(np.ascontiguousarray(x).view(np.float32)), n, p(spec), cols)
        mag = np.abs(spec.view(np.complex64))
        if 2 in types[:cnt]:  # the wideband filter zeroes |.| >= 20
            assert np.min(np.abs(mag - 20.0)) > 0.02, (name, np.min(np.abs(mag - 20.0)))
        out[f"{name}_in"] = x
        out[f"{name}_out"] = iq.view(np.complex64)
        out[f"{name}_fs"] = np.array(fs)
        out[f"{name}_types"] = types[:cnt]
        out[f"{name}_bins"] = bins[:cnt]
        out[f"{name}_freqs"] = freqs[:cnt]
        out[f"{name}_jn"] = jn[:cnt]
        if name == "tone":
            out["stft_cols"] = spec.view(np.complex64).reshape(cols, 128)
            syn = np.zeros(2 * (128 + (cols - 1) * 32), np.float32)
            lib.ref_istft_f32(p(spec), cols, p(syn))
            out["istft"] = syn.view(np.complex64)
    return out


# navigation-symbol streams for the preamble search: (name, message, epochs,
# symbol period ms, preamble period in symbols, seed).  GPS LNAV repeats its
# preamble every subframe (300 bits), the GLONASS time mark every string (2 s).
PREAMBLE_CASES = [
    ("gps_two_subframes", 0, 12000, 20, 300, 11),
    ("gps_inverted", 0, 12000, 20, 300, 12),
    ("gps_odd_length", 0, 6007, 20, 300, 13),
    ("gps_shorter_than_preamble", 0, 100, 20, 300, 14),
    ("gps_zeros", 0, 4000, 20, 300, 15),
    ("glonass_strings", 1, 8000, 10, 200, 16),
    ("glonass_odd_length", 1, 4001, 10, 200, 17),
    ("glonass_shorter_than_preamble", 1, 255, 10, 200, 19),
]
GPS_PREAMBLE = [1, -1, -1, -1, 1, -1, 1, 1]
GLONASS_PREAMBLE = [-1, -1, -1, -1, -1, 1, 1, 1, -1, -1, 1, -1, -1, -1, 1, -1, 1, -1, 1, 1,
                    1, 1, -1, 1, 1, -1, 1, -1, -1, 1, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1]


def preamble_input(name: str, message: int, n: int, period_ms: int, every: int, seed: int) -> np.ndarray:
    """Prompt I (int8 steps) of a channel carrying the message: random symbols
    with the preamble every `every` symbols from a random start, noise, a few
    exact zeros (the search's `> 0` test)."""
    rng = np.random.default_rng(seed)
    pre = np.array(GLONASS_PREAMBLE if message == 1 else GPS_PREAMBLE)
    n_sym = -(-n // period_ms)
    sym = rng.choice([-1, 1], n_sym)
    for s in range(int(rng.integers(0, every)), n_sym - len(pre), every):
        sym[s:s + len(pre)] = pre
    if "shorter" in name and message == 1:
        # the prompt is the cut preamble itself, rotated: the circular
        # filter finds it across the wrap
        sym = np.roll(pre[:n_sym], int(rng.integers(1, n_sym)))
    if "inverted" in name:
        sym = -sym
    x = np.repeat(sym, period_ms)[:n] * 40 + rng.normal(0, 12, n)
    if "zeros" in name:
        x[:] = 0
    x = np.clip(np.rint(x), -127, 127)
    x[rng.integers(0, n, max(1, n // 500))] = 0
    return x.astype(np.int8)


def preamble(lib) -> dict[str, np.ndarray]:
    """The reference's own matched filter + |.| (ref_preamble_filter_f32) over
    sign(prompt I); candidates = epochs above the reference's threshold."""
    out = {}
    for name, message, n, period_ms, every, seed in PREAMBLE_CASES:
        x = preamble_input(name, message, n, period_ms, every, seed)
        xf = x.astype(np.float32)
        y = np.zeros(n, np.float32)
        lib.ref_preamble_filter_f32(p(xf), n, message, p(y))
        threshold = 370 if message == 1 else 153
        idx = np.flatnonzero(y > threshold).astype(np.int32)
        # |y| is twice an integer correlation: far from the threshold
        margin = np.min(np.abs(y - threshold))
        assert margin > 0.5, (name, margin)
        out[f"{name}/prompt_i"] = x
        out[f"{name}/message"] = np.int32(message)
        out[f"{name}/indexes"] = idx
        out[f"{name}/peak"] = np.float32(y.max())
    # CalculateSnr's sigma: the reference's SequentialMeanStdDev over a prompt Q
    q = np.random.default_rng(18).normal(3.0, 40.0, 2000).astype(np.float32)
    mean, sigma = C.c_float(), C.c_float()
    lib.ref_mean_std_f32(p(q), q.size, C.byref(mean), C.byref(sigma))
    out["sigma/prompt_q"] = q
    out["sigma/value"] = np.float32(sigma.value)
    return out


TRACK_FS = 4e6
TRACK_MS = 160


def track(lib) -> dict[str, np.ndarray]:
    """The reference's own tracking arithmetic on a seeded capture (int8 I/Q,
    4 MHz, 160 ms): three GPS L1 C/A channels and one Galileo E1B channel
    (4 ms code period), each started from an acquisition-like state (code
    phase to the sample, Doppler to the 50 Hz grid) and run through
    ref_track_f32 (TrackSingleSatellite with the reference's TableMixer,
    UpdatePhase, CorrelateSplit, Pll, Dll), and AddSignalImpl's refinement
    (ref_refine_f32) from a code phase 3 samples off."""
    d, vp, sz, i = C.c_double, C.c_void_p, C.c_size_t, C.c_int
    lib.ref_track_f32.argtypes = [vp, sz, i, vp, sz, i, d, d, d, d, vp]
    lib.ref_refine_f32.argtypes = [vp, sz, i, i, d, d, d, vp]
    fix = np.load(HERE / "codes.npz")
    ca, e1b = unpack(fix, "gps_l1ca"), unpack(fix, "galileo_e1b")
    rng = np.random.default_rng(31)
    chans = [dict(signal=0, prn=3, chips=ca[3], rate=1.023e6, cn0=47.0, data=50.0),
             dict(signal=0, prn=11, chips=ca[11], rate=1.023e6, cn0=44.0, data=50.0),
             dict(signal=0, prn=24, chips=ca[24], rate=1.023e6, cn0=41.0, data=50.0),
             dict(signal=6, prn=7, chips=e1b[7], rate=2.046e6, cn0=46.0, data=250.0)]
    ems = []
    for ch in chans:
        ch["code_phase_chips"] = rng.uniform(0, len(ch["chips"]))
        ch["doppler"] = rng.uniform(-3500, 3500)
        ems.append(signals.Emitter(ch["chips"], ch["rate"], ch["code_phase_chips"], ch["doppler"], ch["cn0"], ch["data"],
                                   rng.uniform(0, 2 * np.pi)))
    n = int(TRACK_FS * TRACK_MS / 1000)
    raw = signals.synthesize(ems, TRACK_FS, n, 20.0, "ci8", 32)
    x = raw.astype(np.float32)
    x = np.ascontiguousarray((x[:, 0] + 1j * x[:, 1]).astype(np.complex64))
    spm = int(TRACK_FS / 1000)
    out = {"samples": raw, "fs": np.float64(TRACK_FS)}
    for k, ch in enumerate(chans):
        period_ms = int(round(len(ch["chips"]) / ch["rate"] * 1000))
        cp = float(round(ch["code_phase_chips"] / ch["rate"] * TRACK_FS % (period_ms * spm)))
        cf = round(ch["doppler"] / 50.0) * 50.0
        full = np.zeros(3 * period_ms * spm, np.float32)
        rep = np.ascontiguousarray(np.tile(ch["chips"], 3).astype(np.float32))
        lib.ref_repeat_upsample(p(rep), rep.size, 1, p(full), full.size)
        res = np.zeros((TRACK_MS, 12))
        lib.ref_track_f32(p(x), spm, TRACK_MS, p(full), full.size, ch["signal"], TRACK_FS, ch["rate"], cp, cf, p(res))
        ref3 = np.zeros(4)
        lib.ref_refine_f32(p(x), x.size, ch["signal"], ch["prn"], TRACK_FS, cp + 3.0, cf, p(ref3))
        pre = f"ch{k}/"
        out[pre + "signal"] = np.int32(ch["signal"])
        out[pre + "prn"] = np.int32(ch["prn"])
        out[pre + "code_frequency"] = np.float64(ch["rate"])
        out[pre + "code_phase"] = np.float64(cp)
        out[pre + "carrier_frequency"] = np.float64(cf)
        out[pre + "track"] = res
        out[pre + "refine_code_phase"] = np.float64(cp + 3.0)
        out[pre + "refine"] = ref3
    out["channels"] = np.int32(len(chans))
    return out


OBS_IF, OBS_POSITION, OBS_TOW_S = 1250.0, 37, 345678


def observables(lib) -> dict[str, np.ndarray]:
    """The reference's Observable (ref_observable_f64: its constructor with
    CalculateSnr, then TimeScale::UpdateScale and UpdatePseudoranges) on the
    three GPS channels' reference tracking histories in track.npz (prompt,
    carrier phase, carrier frequency, code phase per epoch), at an IF of
    1.25 kHz, a preamble at epoch 37 and a time of week of 345678 s."""
    d, vp, sz = C.c_double, C.c_void_p, C.c_size_t
    lib.ref_observable_f64.argtypes = [vp, vp, vp, vp, sz, d, d, sz, sz, vp]
    z = np.load(HERE / "track.npz")
    fs = float(z["fs"])
    out = {"intermediate_frequency": np.float64(OBS_IF), "position": np.int64(OBS_POSITION),
           "tow_s": np.int64(OBS_TOW_S), "channels": np.int32(3)}
    for k in range(3):  # the GPS L1 C/A channels
        tr = z[f"ch{k}/track"]
        piq = np.ascontiguousarray(tr[:, 2:4].astype(np.float32))
        cph, freq, cp = (np.ascontiguousarray(tr[:, j]) for j in (7, 6, 8))
        res = np.zeros((len(tr), 4))
        lib.ref_observable_f64(p(piq), p(cph), p(freq), p(cp), len(tr), fs, OBS_IF, OBS_POSITION, OBS_TOW_S, p(res))
        out[f"ch{k}"] = res
    return out


def main() -> None:
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).resolve().parents[3] / "reference")
    lib = ref_lib(ref_dir)
    if len(sys.argv) > 2:  # regenerate the named fixtures only, e.g. `preamble`
        for name in sys.argv[2:]:
            np.savez_compressed(HERE / f"{name}.npz", **globals()[name](lib))
        return
    c = codes(lib)
    np.savez_compressed(HERE / "codes.npz", **c)
    k = kats(lib, c)
    np.savez_compressed(HERE / "kats.npz", **k)
    a = acquisition(lib, c)
    np.savez_compressed(HERE / "acq_gps_l1_4mhz.npz", **a)
    np.savez_compressed(HERE / "packed.npz", **packed(lib, ref_dir))
    np.savez_compressed(HERE / "jamming.npz", **jamming(lib))
    np.savez_compressed(HERE / "real8.npz", **real8(ref_dir))
    np.savez_compressed(HERE / "iq16.npz", **iq16(ref_dir))
    np.savez_compressed(HERE / "preamble.npz", **preamble(lib))
    np.savez_compressed(HERE / "track.npz", **track(lib))
    np.savez_compressed(HERE / "observables.npz", **observables(lib))
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
