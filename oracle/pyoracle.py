"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() (as the
checker) and bench.py's cpu_baseline / --impl reference arm.  The product
path never imports this module.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    lib = C.CDLL(str(LIB))
    vp, sz, d, i = C.c_void_p, C.c_size_t, C.c_double, C.c_int
    sigs = {
        "orc_table_mixer_f32": [vp, sz, d, d, d],
        "orc_table_mixer_f64": [vp, sz, d, d, d],
        "orc_dft_c2c_f32": [vp, vp, sz, i],
        "orc_dft_c2c_f64": [vp, vp, sz, i],
        "orc_dft_r2c_f32": [vp, vp, sz],
        "orc_prepare_code_spectrum_f32": [vp, sz, i, vp],
        "orc_prepare_code_spectrum_f64": [vp, sz, i, vp],
        "orc_filter_optimized_f32": [vp, sz, vp, i],
        "orc_filter_optimized_f64": [vp, sz, vp, i],
        "orc_abs_f32": [vp, sz, vp],
        "orc_reshape_sum_f32": [vp, sz, sz],
        "orc_reshape_sum_c32": [vp, sz, sz],
        "orc_max_index_f32": [vp, sz],
        "orc_mean_std_f32": [vp, sz, vp, vp],
        "orc_mean_std_f64": [vp, sz, vp, vp],
        "orc_upsample_f32": [vp, sz, vp, sz],
        "orc_resample_c32": [vp, sz, vp, sz, sz],
        "orc_correlate_f32": [vp, vp, sz, vp],
        "orc_correlate_split_f32": [vp, vp, sz, d, d, vp],
        "orc_acquire_f32": [vp, sz, sz, sz, vp, d, d, d, d, d, i, i, i, i, vp, vp, vp],
        "orc_acquire_f64": [vp, sz, sz, sz, vp, d, d, d, d, d, i, i, i, i, vp, vp, vp],
        "orc_acquire_many_f32": [vp, sz, sz, sz, vp, sz, d, d, d, d, d, i, i, i, i, i, vp],
        "orc_fse_baseline_f32": [vp, sz, sz, sz, vp, sz, d, d, d, i, vp],
        "orc_stft_f32": [vp, sz, i, i, vp],
        "orc_istft_f32": [vp, sz, i, i, vp],
        "orc_jamming_process_f32": [vp, sz, d, i, vp, vp, vp, vp, i],
    }
    for name, args in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = None
    lib.orc_reshape_sum_f32.restype = i
    lib.orc_reshape_sum_c32.restype = i
    lib.orc_max_index_f32.restype = sz
    lib.orc_resample_c32.restype = sz
    lib.orc_stft_f32.restype = sz
    lib.orc_jamming_process_f32.restype = i
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data


REC_FIELDS = ("level", "sigma", "code_offset", "doppler", "index", "doppler_bin", "snr", "mean", "std")


def table_mix(x: np.ndarray, fs: float, f: float, phase: float = 0.0) -> np.ndarray:
    y = np.array(x, copy=True)
    fn = load().orc_table_mixer_f64 if y.dtype == np.complex128 else load().orc_table_mixer_f32
    fn(_p(y), y.size, fs, f, phase)
    return y


def acquire(iq_complex: np.ndarray, n: int, k_blocks: int, code: np.ndarray, fs: float, range_hz: float, step_hz: float,
            if_freq: float = 0.0, ratio: float = 1.0, reshape: bool = False, coherent: bool = True, stat: int = 0,
            spectrum_mode: int = 0, double: bool = False, grid: bool = False):
    """ProcessBpsk restated (oracle.cpp Acquire).  iq_complex: complex samples."""
    lib = load()
    if double:
        x = np.ascontiguousarray(iq_complex, np.complex128)
        c = np.ascontiguousarray(code, np.float64)
        fn = lib.orc_acquire_f64
    else:
        x = np.ascontiguousarray(iq_complex, np.complex64)
        c = np.ascontiguousarray(code, np.float32)
        fn = lib.orc_acquire_f32
    rec = np.zeros(9)
    nbins = len(doppler_grid(range_hz, step_hz))
    g = np.zeros((nbins, 4)) if grid else None
    fn(_p(x), x.size, n, k_blocks, _p(c), fs, range_hz, step_hz, if_freq, ratio, 1 if reshape else 0, 1 if coherent else 0,
       stat, spectrum_mode, _p(rec), _p(g), None)
    out = dict(zip(REC_FIELDS, rec))
    if grid:
        return out, g
    return out


def acquire_many(iq_complex: np.ndarray, n: int, k_blocks: int, codes: np.ndarray, fs: float, range_hz: float,
                 step_hz: float, threads: int = 1, reshape: bool = False, coherent: bool = True, stat: int = 0,
                 spectrum_mode: int = 0) -> np.ndarray:
    lib = load()
    x = np.ascontiguousarray(iq_complex, np.complex64)
    c = np.ascontiguousarray(codes, np.float32)
    recs = np.zeros((c.shape[0], 9))
    lib.orc_acquire_many_f32(_p(x), x.size, n, k_blocks, _p(c), c.shape[0], fs, range_hz, step_hz, 0.0, 1.0,
                             1 if reshape else 0, 1 if coherent else 0, stat, spectrum_mode, threads, _p(recs))
    return recs


def fse_baseline(iq_complex: np.ndarray, n: int, k_blocks: int, codes: np.ndarray, fs: float, range_hz: float,
                 step_hz: float, threads: int = 1) -> np.ndarray:
    """The CPU baseline: acquire_many with float transforms (FftT<float>)."""
    lib = load()
    x = np.ascontiguousarray(iq_complex, np.complex64)
    c = np.ascontiguousarray(codes, np.float32)
    recs = np.zeros((c.shape[0], 9))
    lib.orc_fse_baseline_f32(_p(x), x.size, n, k_blocks, _p(c), c.shape[0], fs, range_hz, step_hz, threads, _p(recs))
    return recs


def doppler_grid(range_hz: float, step_hz: float) -> list[float]:
    out, d = [], -range_hz
    while d <= range_hz:
        out.append(d)
        d += step_hz
    return out


def upsample(code: np.ndarray, samples: int) -> np.ndarray:
    code = np.ascontiguousarray(code, np.float32)
    out = np.empty(samples, np.float32)
    load().orc_upsample_f32(_p(code), code.size, _p(out), samples)
    return out


def resample(x: np.ndarray, new_fs: int, old_fs: int) -> np.ndarray:
    import math
    x = np.ascontiguousarray(x, np.complex64)
    lcm = new_fs * old_fs // math.gcd(new_fs, old_fs)
    up = lcm * x.size // old_fs
    out = np.empty(up // (lcm // new_fs) + 2, np.complex64)
    n = load().orc_resample_c32(_p(x), x.size, _p(out), new_fs, old_fs)
    return out[:n].copy()


TRACK_FIELDS = 21


def track(iq_complex: np.ndarray, spm: int, n_epochs: int, chips: np.ndarray, fs: float, code_frequency: float,
          code_phase: float, carrier_frequency: float, carrier_phase: float = 0.0, early_late: float = 0.25,
          very_early_late: float = 0.5, pll_bw: float = 25.0, dll_bw: float = 0.7, fll_bw: float = 250.0,
          nco_mode: int = 0) -> np.ndarray:
    """FP64 restatement of one tracking channel (track_oracle.cpp); rows of
    VE, E, P, L, VL (re, im), carrier_frequency, carrier_phase, code_phase,
    code_frequency, phase_error, code_error.  nco_mode 1: the reference's
    per-epoch 32-bit TableMixer NCO and radian carrier phase."""
    lib = load()
    fn = lib.orc_track_f64
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = None
    x = np.ascontiguousarray(iq_complex, np.complex64)
    c = np.ascontiguousarray(chips, np.float32)
    cfg = np.array([early_late, very_early_late, pll_bw, dll_bw, fll_bw, 1e-3, float(nco_mode)])
    ch = np.array([fs, code_frequency, float(len(c)), code_phase, carrier_frequency, carrier_phase])
    out = np.zeros((n_epochs, TRACK_FIELDS))
    fn(x.ctypes.data, spm, n_epochs, c.ctypes.data, len(c), cfg.ctypes.data, ch.ctypes.data, out.ctypes.data)
    return out


def track_taps(iq_epoch: np.ndarray, chips: np.ndarray, fs: float, code_frequency: float, code_phase: float,
               carrier_frequency: float, carrier_phase: float, early_late: float = 0.25,
               very_early_late: float = 0.5, nco_mode: int = 0) -> np.ndarray:
    """Open-loop taps of one epoch for a given NCO state (orc_track_taps_f64):
    10 values (VE, E, P, L, VL re/im) + 5 minor partial magnitudes."""
    lib = load()
    fn = lib.orc_track_taps_f64
    d = C.c_double
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_int, d, d, d, d, d, d, d, d, C.c_int, C.c_void_p]
    fn.restype = None
    x = np.ascontiguousarray(iq_epoch, np.complex64)
    c = np.ascontiguousarray(chips, np.float32)
    out = np.zeros(15)
    fn(x.ctypes.data, x.size, c.ctypes.data, len(c), fs, code_frequency, float(len(c)), code_phase, carrier_frequency,
       carrier_phase, early_late, very_early_late, nco_mode, out.ctypes.data)
    return out


def bbp_epoch_bytes(fs: float) -> int:
    """Bytes per 1 ms BBP DDC epoch (signal_parameters.hpp:78-85)."""
    words = fs / 1e3 * 4 / 64 + 1
    b = int(words / 2) * 2
    if words % 2:
        b += 2
    return b * 8


def unpack_bbp(raw: np.ndarray, fs: float) -> np.ndarray:
    """BBP DDC epochs -> complex (helpers/BbpPackedSpan.hpp, signal_parameters.hpp:234-246):
    skip each epoch's 8-byte header; byte s/2 holds sample s, imag in bits
    0-1 / 4-5 and real in bits 2-3 / 6-7, each 2-bit field read as (f | 1)."""
    spm = int(fs / 1e3)
    eb = bbp_epoch_bytes(fs)
    ep = raw.reshape(-1, eb)[:, 8:8 + spm // 2].astype(np.uint8)
    out = np.empty((ep.shape[0], spm), np.complex64)
    for half, sh in ((0, 0), (1, 4)):
        im = np.where((ep >> (sh + 1)) & 1, -1.0, 1.0)
        re = np.where((ep >> (sh + 3)) & 1, -1.0, 1.0)
        out[:, half::2] = re + 1j * im
    return out.reshape(-1)


def unpack_nt1065(raw: np.ndarray, channel: int) -> np.ndarray:
    """NT1065 bytes -> real samples (helpers/NtlabPackedSpan.hpp), channel 0..3 at bit offsets 6, 4, 2, 0."""
    b = raw.astype(np.int32) >> (6 - 2 * channel)
    return ((2 * (b & 1) - 1) * (1 + 2 * ((b >> 1) & 1))).astype(np.complex64)


def track_refine(x: np.ndarray, channels: list[dict], codes: list[np.ndarray]):
    """TrackingParameters::AddSignalImpl's refinement (tracking_parameters.hpp:
    297-357) restated: three code periods translated by -carrier_frequency
    (TableMixer), matched-filtered against one code period upsampled,
    zero-padded to three and rotated right by the integer code phase (the
    reference's FFTW filter: one-sided conj code spectrum, FP64 here), |.|
    folded to one code period, first maximum, offset wrapped to +-period / 2,
    accepted when within 1e-6 fs samples of a whole ms.  Returns (accepted,
    offsets, refined code phases, peak levels)."""
    acc, offs, phases, levels = [], [], [], []
    for ch in channels:
        fs = ch["fs"]
        spm = int(fs / 1e3)
        chips = np.asarray(codes[ch["code"]], np.float32)
        period = spm * int(round(len(chips) / ch["code_frequency"] * 1000))
        n = 3 * period
        y = table_mix(np.ascontiguousarray(x[:n], np.complex64), fs, -ch["carrier_frequency"]).astype(np.complex128)
        replica = np.zeros(n, np.float64)
        replica[:period] = upsample(chips, period)
        replica = np.roll(replica, int(ch["code_phase"]))          # std::rotate right by (ptrdiff_t)code_phase
        spec = np.fft.fft(replica)
        spec[n // 2 + 1:] = 0.0                                    # r2c: bins above N/2 stay zero (dft.hpp:37-46)
        mf = np.abs(np.fft.ifft(np.fft.fft(y) * np.conj(spec)) * 2.0)
        folded = mf.reshape(3, period).sum(axis=0)
        off = int(np.argmax(folded))
        if off > period // 2:
            off -= period
        mod = (off + period) % spm
        if mod > spm // 2:
            mod -= spm
        ok = abs(mod) < 1e-6 * fs
        acc.append(1 if ok else 0)
        offs.append(off)
        phases.append(ch["code_phase"] + off if ok else ch["code_phase"])
        levels.append(float(folded.max()))
    return acc, offs, phases, levels


def track_loop(taps: np.ndarray, fs: float, code_frequency: float, code_phase: float, carrier_frequency: float,
               pll_bw: float = 25.0, dll_bw: float = 0.7, fll_bw: float = 250.0) -> np.ndarray:
    """The oracle's loop update alone (orc_track_loop_f64) on given per-epoch
    E, P, L taps (rows of 6: re, im): rows of carrier_frequency, carrier_phase
    (rad), code_phase, code_frequency, phase_error, code_error."""
    lib = load()
    fn = lib.orc_track_loop_f64
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = None
    t = np.ascontiguousarray(taps, np.float64)
    cfg = np.array([pll_bw, dll_bw, fll_bw, 1e-3, fs, code_frequency])
    init = np.array([carrier_frequency, 0.0, code_phase])
    out = np.zeros((t.shape[0], 6))
    fn(t.ctypes.data, t.shape[0], cfg.ctypes.data, init.ctypes.data, out.ctypes.data)
    return out


def stft(x: np.ndarray, window: int = 128, overlap: int = 96) -> np.ndarray:
    """SequentialStft split (math/stft.hpp:42-61): (columns, window) complex64."""
    x = np.ascontiguousarray(x, np.complex64)
    lib = load()
    cols = lib.orc_stft_f32(_p(x), x.size, window, overlap, None)
    out = np.empty((cols, window), np.complex64)
    lib.orc_stft_f32(_p(x), x.size, window, overlap, _p(out))
    return out


def istft(columns: np.ndarray, overlap: int = 96) -> np.ndarray:
    """OverlapAndAdd (math/stft.hpp:63-75)."""
    columns = np.ascontiguousarray(columns, np.complex64)
    n_cols, w = columns.shape
    out = np.empty(w + (n_cols - 1) * (w - overlap), np.complex64)
    load().orc_istft_f32(_p(columns), n_cols, w, overlap, _p(out))
    return out


def jamming(x: np.ndarray, fs: float, suppress: bool = True):
    """JammingDetector::Process (suppress False) or JammingSuppressionEngine::
    Process (antijamming/jse.hpp:89-102) on a copy of x: (detections as
    (type, bin, frequency, J/N) tuples, output samples)."""
    y = np.array(x, np.complex64, copy=True)
    types = np.zeros(64, np.int32)
    bins = np.zeros(64, np.int64)
    freqs = np.zeros(64)
    jn = np.zeros(64)
    cnt = load().orc_jamming_process_f32(_p(y), y.size, fs, 1 if suppress else 0, _p(types), _p(bins), _p(freqs),
                                         _p(jn), 64)
    det = [(int(types[i]), int(bins[i]), float(freqs[i]), float(jn[i])) for i in range(min(cnt, 64))]
    return det, y


NAV_GPS_LNAV, NAV_GLONASS = 0, 1


def preamble_search(prompt_i: np.ndarray, message: int, cap: int = 4096) -> list[int]:
    """FindPreambleGps / Glonass's candidate epochs (obs_oracle.cpp), ascending."""
    fn = load().orc_preamble_search
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_void_p, C.c_int]
    fn.restype = C.c_int
    x = np.ascontiguousarray(prompt_i, np.float32)
    idx = np.zeros(cap, np.int32)
    n = fn(x.ctypes.data, x.size, message, idx.ctypes.data, cap)
    if n > cap:
        raise ValueError(f"{n} candidates, more than cap={cap}")
    return idx[:n].tolist()


def observables(rows: np.ndarray, fs: float, intermediate_frequency: float, carrier_frequency0: float,
                carrier_phase0: float, position: int, correction: float = 0.0) -> np.ndarray:
    """Observable's arithmetic for one channel (obs_oracle.cpp) from its
    tracking rows (TRACK_DTYPE-like record array with taps, carrier_frequency,
    phase_error, code_phase); (n, 4): pseudorange, pseudophase, doppler, snr."""
    fn = load().orc_observables_f64
    d = C.c_double
    fn.argtypes = [C.c_void_p] * 5 + [C.c_size_t, d, d, d, d, C.c_size_t, d, C.c_void_p]
    fn.restype = None
    pi = np.ascontiguousarray(rows["taps"][:, 2, 0], np.float32)
    pq = np.ascontiguousarray(rows["taps"][:, 2, 1], np.float32)
    f = np.ascontiguousarray(rows["carrier_frequency"], np.float64)
    err = np.ascontiguousarray(rows["phase_error"], np.float64)
    cp = np.ascontiguousarray(rows["code_phase"], np.float64)
    out = np.zeros((len(rows), 4))
    fn(pi.ctypes.data, pq.ctypes.data, f.ctypes.data, err.ctypes.data, cp.ctypes.data, len(rows), fs,
       intermediate_frequency, carrier_frequency0, carrier_phase0, position, correction, out.ctypes.data)
    return out
