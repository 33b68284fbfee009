"""Seeded synthetic GNSS baseband generator (numpy).

Stands in for recorded captures: the acquisition benchmark configurations
name signal mixes (visible PRNs, C/N0, Doppler, data bits, AWGN, int8/int16
quantisation) rather than a dataset, so inputs are synthesised from a seed.

Model per emitter: s[n] = A d(t) c(R (t - tau)) exp(j (2 pi f_D t + phi))
with t = n / fs, code c (+-1 chips, BOC already expanded), chip rate R,
data bits d at `data_rate`, amplitude A = sigma sqrt(2 C/N0 / fs) for complex
AWGN of standard deviation sigma per component.  A matched filter against
the local code started at sample 0 peaks at lag tau * fs samples.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Emitter:
    chips: np.ndarray        # +-1 per chip (one code period)
    chip_rate: float         # chips/s
    code_phase: float        # chips of delay tau * R
    doppler: float           # Hz (carrier offset in the sampled band)
    cn0_dbhz: float
    data_rate: float = 50.0  # bits/s (0 = pilot)
    phase: float = 0.0
    tag: object = None
    secondary: np.ndarray | None = None  # +-1 per primary code period (e.g. NH10), repeating


def synthesize(emitters: list[Emitter], fs: float, n: int, noise_sigma: float, sample_type: str, seed: int,
               real_if: bool = False) -> np.ndarray:
    """Returns interleaved int8/int16 I/Q ('ci8'/'ci16', shape (n, 2)), complex64 ('cf32')
    or real int8 ('ri8', shape (n,)).  real_if: emitters already carry their IF
    in `doppler`; the real part is kept (noise of sigma on the real channel)."""
    rng = np.random.default_rng(seed)
    t = np.arange(n, dtype=np.float64) / fs
    acc = np.zeros(n, np.complex128)
    for e in emitters:
        amp = noise_sigma * np.sqrt(2.0 * 10 ** (e.cn0_dbhz / 10.0) / fs)
        pos = (t * e.chip_rate - e.code_phase) % len(e.chips)
        code = e.chips[np.floor(pos).astype(np.int64) % len(e.chips)]
        if e.secondary is not None:
            period = np.floor((t * e.chip_rate - e.code_phase) / len(e.chips)).astype(np.int64)
            code = code * np.asarray(e.secondary, np.float64)[period % len(e.secondary)]
        if e.data_rate > 0:
            bit_off = rng.uniform(0, 1.0 / e.data_rate)
            nbits = int(np.ceil((t[-1] + bit_off) * e.data_rate)) + 2
            bits = rng.choice([-1.0, 1.0], size=nbits)
            data = bits[np.floor((t + bit_off) * e.data_rate).astype(np.int64)]
        else:
            data = 1.0
        acc += amp * data * code * np.exp(1j * (2 * np.pi * e.doppler * t + e.phase))
    if sample_type == "ri8":
        x = np.real(acc) * np.sqrt(2.0) + rng.normal(0, noise_sigma, n)
        return np.clip(np.round(x), -128, 127).astype(np.int8)
    noise = rng.normal(0, noise_sigma, (n, 2))
    iq = np.stack([acc.real, acc.imag], axis=1) + noise
    if sample_type == "ci8":
        return np.clip(np.round(iq), -128, 127).astype(np.int8)
    if sample_type == "ci16":
        return np.clip(np.round(iq), -32768, 32767).astype(np.int16)
    if sample_type == "cf32":
        return (iq[:, 0] + 1j * iq[:, 1]).astype(np.complex64)
    raise ValueError(sample_type)


def boc_expand(chips: np.ndarray) -> np.ndarray:
    """Sine BOC(1,1) half-chips [c, -c] per chip (MemoryCodes::DecodeBoc, MemoryCodes.hpp:33-40)."""
    out = np.empty(2 * len(chips), np.float32)
    out[0::2] = chips
    out[1::2] = -chips
    return out


def gps_l1_config(seed: int, codes: dict[int, np.ndarray], fs: float = 4.0e6, ms: int = 10, visible: int = 6,
                  cn0=(40.0, 48.0), max_doppler: float = 4500.0, sigma: float = 20.0, sample_type: str = "ci8"):
    """GPS L1 C/A at fs (default: 4 MHz, 10 ms, 6 visible of 32, int8)."""
    rng = np.random.default_rng(seed)
    prns = sorted(codes)
    chosen = rng.choice(prns, size=visible, replace=False)
    ems, truth = [], []
    for p in chosen:
        e = Emitter(codes[int(p)], 1.023e6, rng.uniform(0, 1023), rng.uniform(-max_doppler, max_doppler),
                    rng.uniform(*cn0), 50.0, rng.uniform(0, 2 * np.pi), tag=int(p))
        ems.append(e)
        truth.append(dict(prn=int(p), doppler=e.doppler, code_phase_samples=(e.code_phase / 1.023e6 * fs) % (fs / 1e3),
                          cn0=e.cn0_dbhz))
    n = int(round(fs * ms / 1000))
    return synthesize(ems, fs, n, sigma, sample_type, seed + 1000), truth


# Neuman-Hofman 10-bit secondary code of the GPS L5 I5 channel (IS-GPS-705,
# first bit first): one bit per 1 ms primary period.
NH10 = np.array([0, 0, 0, 0, 1, 1, 0, 1, 0, 1], np.int8)


def nh10_mask() -> int:
    """Sign mask of NH10 for ugsdr_code_put: bit s set = period s negated."""
    return int(sum(1 << s for s, b in enumerate(NH10) if b))


def l5_weak_config(seed: int, codes: dict[int, np.ndarray], fs: float = 40e6, if_hz: float = 10e6, ms: int = 200,
                   visible: int = 8, cn0=(30.0, 38.0), max_doppler: float = 4500.0, sigma: float = 20.0):
    """GPS L5I with NH10 at a real IF: real int8 samples at fs, carrier at if_hz
    plus Doppler, code phase uniform over the 10 ms NH period.  Pilot-like
    (no data symbols), so a 10 ms coherent block sees only the NH10 flips."""
    rng = np.random.default_rng(seed)
    prns = sorted(codes)
    chosen = rng.choice(prns, size=visible, replace=False)
    ems, truth = [], []
    sec = 1.0 - 2.0 * NH10
    for p in chosen:
        delay = rng.uniform(0, 10 * 10230)  # chips within the NH period
        dop = rng.uniform(-max_doppler, max_doppler)
        e = Emitter(codes[int(p)], 10.23e6, delay, if_hz + dop, rng.uniform(*cn0), 0.0, rng.uniform(0, 2 * np.pi),
                    tag=int(p), secondary=sec)
        ems.append(e)
        truth.append(dict(prn=int(p), doppler=dop, delay_chips=delay, cn0=e.cn0_dbhz))
    n = int(round(fs * ms / 1000))
    return synthesize(ems, fs, n, sigma, "ri8", seed + 1000, real_if=True), truth
