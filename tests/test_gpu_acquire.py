"""Batched acquisition engine (ugsdr_acquire) against the reference's own
float/double results (golden) and the oracle.

Bars: peak code-phase index and Doppler bin bit-exact; level, mean, sigma
and SNR within 1e-4 relative of the FP64 oracle."""
import numpy as np
import pytest

from conftest import GOLDEN as GOLDEN_DIR, unpack_codes
from ugsdr_gb300 import _lib as L
from ugsdr_gb300 import signals

pytestmark = pytest.mark.gpu
RTOL = 1e-4


def to_complex(raw):
    if raw.ndim == 2:
        f = raw.astype(np.float32)
        return (f[:, 0] + 1j * f[:, 1]).astype(np.complex64)
    return raw.astype(np.complex64)


def stype(raw):
    if raw.dtype == np.complex64:
        return L.SAMPLES_CF32
    if raw.ndim == 1:
        return L.SAMPLES_RI8
    return L.SAMPLES_CI8 if raw.dtype == np.int8 else L.SAMPLES_CI16


def run_engine(ctx, raw, fs, n, k, code_chips, samples_repeat, range_hz, step_hz, **kw):
    sign_masks = kw.pop("sign_masks", [0] * len(code_chips))
    sign_segment = kw.pop("sign_segment", 0)
    mode = kw.get("spectrum_mode", L.SPECTRUM_ONE_SIDED)
    handles = [ctx.code_put(c, n, repeats=samples_repeat, spectrum_mode=mode, sign_mask=m, sign_segment=sign_segment)
               for c, m in zip(code_chips, sign_masks)]
    try:
        job = ctx.make_job(raw, stype(raw), fs, n, k, handles, range_hz, step_hz, **kw)
        return ctx.acquire(job, cells=True)
    finally:
        for h in handles:
            ctx.code_release(h)


def check_vs_oracle(res, oracle_rec, oracle64):
    assert res.index == int(oracle_rec["index"]), (res, oracle_rec)
    assert res.doppler_bin == int(oracle_rec["doppler_bin"])
    assert res.doppler == pytest.approx(oracle_rec["doppler"], abs=1e-9)
    for f in ("level", "mean", "std", "snr", "sigma"):
        assert abs(getattr(res, f) - oracle64[f]) <= RTOL * abs(oracle64[f]), (f, getattr(res, f), oracle64[f])


def test_gps_l1_4mhz_matches_reference(ctx, acq_golden, golden_codes):
    """Full-size GPS L1 C/A search: int8 IQ, 4 MHz, 1 ms x 10 blocks, 21 Doppler bins."""
    ca = unpack_codes(golden_codes, "gps_l1ca")
    raw = acq_golden["acq_raw"]
    prns = acq_golden["acq_prns"]
    res, cells = run_engine(ctx, raw, 4e6, 4000, 10, [ca[p] for p in prns], 1, 5000, 500)
    for r, rec, rec64 in zip(res, acq_golden["acq_rec"], acq_golden["acq_rec64"]):
        assert r.index == int(rec[4]) and r.doppler_bin == int(rec[5])
        assert abs(r.level - rec64[0]) <= RTOL * rec64[0]
        assert abs(r.sigma - rec64[1]) <= RTOL * rec64[1]
        assert abs(r.snr - rec64[6]) <= RTOL * rec64[6]
        assert r.n_doppler == 21
    # the visible satellites are found at their true code phase
    truth = {int(t[0]): t for t in acq_golden["acq_truth"]}
    for p, r in zip(prns, res):
        if int(p) in truth:
            assert abs(r.index - truth[int(p)][2]) <= 1.0
            assert abs(r.doppler - truth[int(p)][1]) <= 250.0 + 1e-9


@pytest.mark.parametrize("mode,stat", [(L.SPECTRUM_TWO_SIDED, L.STAT_ABS), (L.SPECTRUM_ONE_SIDED, L.STAT_ABS2)])
def test_modes_vs_oracle(ctx, oracle, acq_golden, golden_codes, mode, stat):
    ca = unpack_codes(golden_codes, "gps_l1ca")
    raw = acq_golden["acq_raw"][:16000]
    x = to_complex(raw)
    prns = [int(p) for p in acq_golden["acq_prns"][:3]]
    res, _ = run_engine(ctx, raw, 4e6, 4000, 4, [ca[p] for p in prns], 1, 5000, 500, statistic=stat, spectrum_mode=mode)
    for p, r in zip(prns, res):
        code = oracle.upsample(ca[p], 4000)
        o32 = oracle.acquire(x, 4000, 4, code, 4e6, 5000, 500, stat=stat, spectrum_mode=mode)
        o64 = oracle.acquire(x, 4000, 4, code, 4e6, 5000, 500, stat=stat, spectrum_mode=mode, double=True)
        check_vs_oracle(r, o32, o64)


@pytest.mark.parametrize("coherent", [True, False])
def test_fold_4ms_vs_oracle(ctx, oracle, acq_golden, golden_codes, coherent):
    """Reference layout: 4 ms code (RepeatCodeNTimes 4) folded to 1 ms (fse.hpp:201-220, 295-296)."""
    ca = unpack_codes(golden_codes, "gps_l1ca")
    raw = acq_golden["acq_raw"][:32000]
    x = to_complex(raw)
    prns = [int(p) for p in acq_golden["acq_prns"][:2]]
    res, _ = run_engine(ctx, raw, 4e6, 16000, 2, [ca[p] for p in prns], 4, 3000, 500, fold_samples=4000,
                        fold_coherent=coherent)
    for p, r in zip(prns, res):
        code = oracle.upsample(np.tile(ca[p], 4), 16000)
        o32 = oracle.acquire(x, 16000, 2, code, 4e6, 3000, 500, reshape=True, coherent=coherent)
        o64 = oracle.acquire(x, 16000, 2, code, 4e6, 3000, 500, reshape=True, coherent=coherent, double=True)
        check_vs_oracle(r, o32, o64)


def test_odd_radix_2046_int16(ctx, oracle, golden_codes):
    """2.046 MHz (N = 2046 = 2*3*11*31), int16 IQ."""
    ca = unpack_codes(golden_codes, "gps_l1ca")
    codes = {i: ca[i] for i in range(8)}
    raw, truth = signals.gps_l1_config(seed=5, codes=codes, fs=2.046e6, ms=6, visible=3, sample_type="ci16", cn0=(46, 50))
    x = to_complex(raw)
    prns = [t["prn"] for t in truth]
    res, _ = run_engine(ctx, raw, 2.046e6, 2046, 6, [ca[p] for p in prns], 1, 5000, 1000)
    for p, r in zip(prns, res):
        code = oracle.upsample(ca[p], 2046)
        check_vs_oracle(r, oracle.acquire(x, 2046, 6, code, 2.046e6, 5000, 1000),
                        oracle.acquire(x, 2046, 6, code, 2.046e6, 5000, 1000, double=True))


@pytest.mark.parametrize("mode", [L.SPECTRUM_ONE_SIDED, L.SPECTRUM_TWO_SIDED])
def test_large_50000_vs_oracle(ctx, oracle, golden_codes, mode):
    """50 MHz, 1 ms blocks: N = 50,000 (four-step path), int16 IQ; one-sided
    spectra run the row stage's pruned gather (Z's upper half is zero),
    two-sided ones the full one."""
    ca = unpack_codes(golden_codes, "gps_l1ca")
    codes = {i: ca[i] for i in range(4)}
    raw, truth = signals.gps_l1_config(seed=9, codes=codes, fs=50e6, ms=2, visible=2, sample_type="ci16", cn0=(48, 50),
                                       max_doppler=1000)
    x = to_complex(raw)
    prns = [t["prn"] for t in truth]
    res, _ = run_engine(ctx, raw, 50e6, 50000, 2, [ca[p] for p in prns], 1, 1000, 500, spectrum_mode=mode)
    for p, r, t in zip(prns, res, truth):
        code = oracle.upsample(ca[p], 50000)
        check_vs_oracle(r, oracle.acquire(x, 50000, 2, code, 50e6, 1000, 500, spectrum_mode=mode),
                        oracle.acquire(x, 50000, 2, code, 50e6, 1000, 500, spectrum_mode=mode, double=True))
        assert abs(r.index - t["code_phase_samples"]) <= 0.1 * 50e6 / 1.023e6  # within 0.1 chip


def test_galileo_e1b_200000_sign_permutation(ctx, oracle, golden_codes):
    """E1B BOC(1,1), 4 ms coherent at 50 MHz: N = 200,000, per-ms sign mask (fse.hpp:374-388)."""
    e1b = unpack_codes(golden_codes, "galileo_e1b")
    em = signals.Emitter(e1b[3], 2.046e6, 1234.5, 250.0, 50.0, data_rate=0.0)
    raw = signals.synthesize([em], 50e6, 200000, 20.0, "ci16", seed=3)
    x = to_complex(raw)
    res, _ = run_engine(ctx, raw, 50e6, 200000, 1, [e1b[3], e1b[3]], 1, 500, 250, sign_masks=[0, 0b1000],
                        sign_segment=50000)
    for mask, r in zip([0, 0b1000], res):
        code = oracle.upsample(e1b[3], 200000)
        code[150000:] *= -1 if mask else 1
        check_vs_oracle(r, oracle.acquire(x, 200000, 1, code, 50e6, 500, 250),
                        oracle.acquire(x, 200000, 1, code, 50e6, 500, 250, double=True))
    assert abs(res[0].index - 1234.5 / 2.046e6 * 50e6) <= 0.2 * 50e6 / 2.046e6


def test_l5_204600_noncoherent_fold(ctx, oracle, golden_codes):
    """L5I at 20.46 MHz, 10 ms coherent (N = 204,600 = 2^3*3*5^2*11*31), complex fold to 1 ms."""
    l5 = unpack_codes(golden_codes, "gps_l5i")
    em = signals.Emitter(l5[4], 10.23e6, 5000.0, -200.0, 52.0, data_rate=0.0)
    raw = signals.synthesize([em], 20.46e6, 204600, 20.0, "ci8", seed=4)
    x = to_complex(raw)
    res, _ = run_engine(ctx, raw, 20.46e6, 204600, 1, [l5[4]], 10, 400, 200, fold_samples=20460, fold_coherent=False)
    code = oracle.upsample(np.tile(l5[4], 10), 204600)
    check_vs_oracle(res[0], oracle.acquire(x, 204600, 1, code, 20.46e6, 400, 200, reshape=True, coherent=False),
                    oracle.acquire(x, 204600, 1, code, 20.46e6, 400, 200, reshape=True, coherent=False, double=True))
    assert abs(res[0].index - 5000.0 * 2) <= 0.2 * 2


def test_batch_equals_single(ctx, acq_golden, golden_codes):
    ca = unpack_codes(golden_codes, "gps_l1ca")
    raw = acq_golden["acq_raw"]
    hs = [ctx.code_put(ca[p], 4000) for p in acq_golden["acq_prns"][:4]]
    try:
        j1 = ctx.make_job(raw, L.SAMPLES_CI8, 4e6, 4000, 10, hs, 5000, 500)
        j2 = ctx.make_job(raw[:20000], L.SAMPLES_CI8, 4e6, 4000, 5, hs[:2], 2000, 250)
        single = [ctx.acquire(j1), ctx.acquire(j2)]
        batch = ctx.acquire_batch([j1, j2])
        for s, b in zip(single, batch):
            for x, y in zip(s, b):
                assert (x.index, x.doppler_bin, x.level, x.snr) == (y.index, y.doppler_bin, y.level, y.snr)
    finally:
        for h in hs:
            ctx.code_release(h)


def test_device_resident_samples(ctx, acq_golden, golden_codes):
    torch = pytest.importorskip("torch")
    ca = unpack_codes(golden_codes, "gps_l1ca")
    raw = acq_golden["acq_raw"]
    dev = torch.from_numpy(raw.copy()).cuda()
    torch.cuda.synchronize()
    hs = [ctx.code_put(ca[p], 4000) for p in acq_golden["acq_prns"][:2]]
    try:
        host = ctx.acquire(ctx.make_job(raw, L.SAMPLES_CI8, 4e6, 4000, 10, hs, 5000, 500))
        devr = ctx.acquire(ctx.make_job(dev.data_ptr(), L.SAMPLES_CI8, 4e6, 4000, 10, hs, 5000, 500,
                                        n_samples=raw.shape[0], on_device=True))
        for a, b in zip(host, devr):
            assert (a.index, a.doppler_bin, a.level) == (b.index, b.doppler_bin, b.level)
    finally:
        for h in hs:
            ctx.code_release(h)


def test_invalid_jobs(ctx, acq_golden, golden_codes):
    ca = unpack_codes(golden_codes, "gps_l1ca")
    raw = acq_golden["acq_raw"]
    h = ctx.code_put(ca[0], 4000)
    try:
        with pytest.raises(L.UgsdrError) as e:  # more blocks than samples
            ctx.acquire(ctx.make_job(raw[:8000], L.SAMPLES_CI8, 4e6, 4000, 3, [h], 5000, 500))
        assert e.value.status == L.E_INVALID
        with pytest.raises(L.UgsdrError) as e:  # code length differs from the block
            ctx.acquire(ctx.make_job(raw, L.SAMPLES_CI8, 4e6, 8000, 2, [h], 5000, 500))
        with pytest.raises(L.UgsdrError) as e:  # unknown handle
            ctx.acquire(ctx.make_job(raw, L.SAMPLES_CI8, 4e6, 4000, 2, [h + 999], 5000, 500))
        assert e.value.status == L.E_NOT_FOUND
        with pytest.raises(L.UgsdrError):  # fold that does not divide the block (reshape_and_sum.hpp:15-18)
            ctx.acquire(ctx.make_job(raw, L.SAMPLES_CI8, 4e6, 4000, 2, [h], 5000, 500, fold_samples=3000))
        with pytest.raises(L.UgsdrError):  # prime factor above 31
            ctx.code_put(ca[0], 4000 * 37)
    finally:
        ctx.code_release(h)
    with pytest.raises(L.UgsdrError) as e:
        ctx.code_release(h)
    assert e.value.status == L.E_NOT_FOUND


@pytest.mark.parametrize("budget_mb", ["1", "8"])
def test_doppler_chunking_same_results(ctx, acq_golden, golden_codes, monkeypatch, budget_mb):
    """A small spectra budget splits the Doppler grid into several launches
    (small path: 4000-point blocks; large path: 50,000-point blocks); results
    must not change."""
    ca = unpack_codes(golden_codes, "gps_l1ca")
    raw = acq_golden["acq_raw"]
    hs = [ctx.code_put(ca[p], 4000) for p in acq_golden["acq_prns"][:3]]
    raw50 = signals.gps_l1_config(seed=9, codes={i: ca[i] for i in range(4)}, fs=50e6, ms=2, visible=2,
                                  sample_type="ci16")[0]
    hl = [ctx.code_put(ca[p], 50000) for p in range(3)]
    try:
        jobs = [ctx.make_job(raw, L.SAMPLES_CI8, 4e6, 4000, 10, hs, 5000, 500),
                ctx.make_job(raw50, L.SAMPLES_CI16, 50e6, 50000, 2, hl, 2000, 500)]
        whole = [ctx.acquire(j, cells=True)[1] for j in jobs]
        monkeypatch.setenv("UGSDR_SPECTRA_BUDGET_MB", budget_mb)
        chunked = [ctx.acquire(j, cells=True)[1] for j in jobs]
        for a, b in zip(whole, chunked):
            np.testing.assert_array_equal(a["index"], b["index"])
            np.testing.assert_allclose(a["level"], b["level"], rtol=1e-6)
    finally:
        for h in hs + hl:
            ctx.code_release(h)


def test_large_368280_runtime_plan(ctx, oracle, golden_codes):
    """GPS L1 at 20.46 MHz, 18 ms coherent: N = 368,280 = 594 x 620 runs the
    runtime-planned four-step kernels, and its scratch regions are not
    multiples of 256 bytes (the layout must round every region the same way
    when sizing and when carving)."""
    ca = unpack_codes(golden_codes, "gps_l1ca")
    em = signals.Emitter(ca[2], 1.023e6, 321.5, 300.0, 50.0, data_rate=0.0)
    raw = signals.synthesize([em], 20.46e6, 368280, 20.0, "ci16", seed=15)
    x = to_complex(raw)
    res, _ = run_engine(ctx, raw, 20.46e6, 368280, 1, [ca[2]], 18, 300, 300)
    code = oracle.upsample(np.tile(ca[2], 18), 368280)
    o32 = oracle.acquire(x, 368280, 1, code, 20.46e6, 300, 300)
    o64 = oracle.acquire(x, 368280, 1, code, 20.46e6, 300, 300, double=True)
    # 18 repetitions of a 1 ms code without data: 18 equal peaks, one per
    # period, so rounding may pick any of them; the peak is exact modulo 1 ms
    r = res[0]
    assert r.index % 20460 == int(o32["index"]) % 20460 and r.doppler_bin == int(o32["doppler_bin"])
    for f in ("level", "mean", "std", "snr", "sigma"):
        assert abs(getattr(r, f) - o64[f]) <= RTOL * abs(o64[f]), (f, getattr(r, f), o64[f])
    assert abs(r.index % 20460 - 321.5 * 20) <= 2


@pytest.mark.parametrize("fs,ms,k", [(4e6, 4, 2), (10.23e6, 12, 1), (6.144e6, 16, 1), (12.5e6, 8, 1), (50e6, 20, 1)])
def test_runtime_four_step_sizes_vs_oracle(ctx, oracle, golden_codes, fs, ms, k):
    """Block sizes of the served mix's kind on the runtime four-step splits
    (16,000; 122,760; 98,304; 100,000) and on runtime columns with the
    compile-time 1000-point rows (1,000,000 = 1000 x 1000), a Galileo
    E1B BOC(1,1) code repeated over whole 4 ms periods: peak bin exact, peak
    index exact modulo the code period (the replica repeats), levels within
    the FP64 bar."""
    chips = unpack_codes(golden_codes, "galileo_e1b")[7]  # 8184 BOC half-chips per 4 ms
    n = int(round(fs * ms / 1000))
    reps = max(1, ms // 4)
    samples_per_period = n // reps
    em = signals.Emitter(chips, 2.046e6, 1234.25, 250.0, 60.0, data_rate=0.0)  # no half-sample delays
    raw = signals.synthesize([em], fs, n * k, 20.0, "ci16", seed=int(fs) % 97 + ms)
    x = to_complex(raw)
    res, _ = run_engine(ctx, raw, fs, n, k, [chips], reps, 500, 250)
    code = oracle.upsample(np.tile(chips, reps), n)
    o32 = oracle.acquire(x, n, k, code, fs, 500, 250)
    o64 = oracle.acquire(x, n, k, code, fs, 500, 250, double=True)
    r = res[0]
    assert r.doppler_bin == int(o32["doppler_bin"])
    assert r.index % samples_per_period == int(o32["index"]) % samples_per_period
    for f in ("level", "mean", "std", "snr", "sigma"):
        assert abs(getattr(r, f) - o64[f]) <= RTOL * abs(o64[f]), (f, getattr(r, f), o64[f])


@pytest.mark.parametrize("new_fs", [9.548e6, 1.736e6, 38.192e6])
def test_real_8_capture_known_answer(ctx, oracle, golden_codes, new_fs):
    """The reference's real-signal acquisition test (test/integration_tests.cpp
    :406-409, 253-263, 237-241) on its real_8.bin capture (first 4 ms: real
    int8 at 38.192 MHz, centre 9.55 MHz above L1): the front end translates
    by +9.55 MHz at the input rate (dfe.hpp:185, 199) and resamples to the
    rate AdjustSamplingRate picks for the FSE targets 8.192 / 2.048 / 40.96
    MHz (fse.hpp:222-240: 9.548, 1.736, 38.192 MHz); 32 GPS C/A codes of
    4 ms folded to 1 ms, +-6 kHz in 200 Hz.  The known answer passes when
    >= 4 of its 8 satellites are found within 400 Hz; peaks of those
    satellites equal the oracle's (at the two lower rates)."""
    z = np.load(GOLDEN_DIR / "real8.npz")
    raw = z["samples"]
    fs, f_if = float(z["fs"]), float(z["if_hz"])
    ca = unpack_codes(golden_codes, "gps_l1ca")
    n = int(round(new_fs * 4 / 1000))
    svs = list(range(32))
    handles = [ctx.code_put(ca[sv], n, repeats=4) for sv in svs]
    try:
        job = ctx.make_job(raw, L.SAMPLES_RI8, new_fs, n, 1, handles, 6000, 200, n_samples=raw.size,
                           input_sampling_rate=fs, frontend_frequency=f_if, code_offset_ratio=fs / new_fs,
                           fold_samples=n // 4, fold_coherent=True)
        res = ctx.acquire(job)
    finally:
        for h in handles:
            ctx.code_release(h)
    found = [sv for sv, dop, _ in z["kat"]
             if res[int(sv)].snr > 3.3 and abs(res[int(sv)].doppler - dop) <= 400]
    assert len(found) >= 4, found  # the reference's rule
    assert len(found) == 8, found  # all are found (lowest SNR 3.7, at 1.736 MHz)
    if new_fs == fs:
        return  # the oracle's 152,768-point search is minutes of CPU
    y = oracle.table_mix(raw.astype(np.complex64), fs, f_if)
    y = oracle.resample(y, int(new_fs), int(fs))[:n]
    check = found if new_fs < 5e6 else found[:4]
    for sv in check:
        code = oracle.upsample(np.tile(ca[int(sv)], 4), n)
        o32 = oracle.acquire(y, n, 1, code, new_fs, 6000, 200, reshape=True, coherent=True)
        o64 = oracle.acquire(y, n, 1, code, new_fs, 6000, 200, reshape=True, coherent=True, double=True)
        check_vs_oracle(res[int(sv)], o32, o64)


def test_iq_16_capture_search(ctx, oracle, golden_codes):
    """The reference's iq_16_plus_16 acquisition test (test/integration_tests
    .cpp:401-404: 4 MHz int16 I/Q on L1, +-15 kHz, non-empty result; the FSE
    keeps 4 MHz, fse.hpp:222-240): 32 GPS C/A codes of 4 ms folded to 1 ms.
    The result is non-empty, and the clear detections (SNR > 4) equal the
    oracle's peaks."""
    z = np.load(GOLDEN_DIR / "iq16.npz")
    raw = z["samples"]
    fs = float(z["fs"])
    ca = unpack_codes(golden_codes, "gps_l1ca")
    n = 16000
    handles = [ctx.code_put(ca[sv], n, repeats=4) for sv in range(32)]
    try:
        job = ctx.make_job(raw, L.SAMPLES_CI16, fs, n, 1, handles, 15000, 200, fold_samples=4000, fold_coherent=True)
        res = ctx.acquire(job)
    finally:
        for h in handles:
            ctx.code_release(h)
    assert any(r.snr > 3.3 for r in res)
    x = to_complex(raw)
    clear = [sv for sv in range(32) if res[sv].snr > 4.0]
    assert len(clear) >= 4, clear
    for sv in clear:
        code = oracle.upsample(np.tile(ca[sv], 4), n)
        o32 = oracle.acquire(x, n, 1, code, fs, 15000, 200, reshape=True, coherent=True)
        o64 = oracle.acquire(x, n, 1, code, fs, 15000, 200, reshape=True, coherent=True, double=True)
        check_vs_oracle(res[sv], o32, o64)


def test_maximum_block_size_2_24(ctx, oracle, golden_codes):
    """The largest block the engine takes (2^24 = 16,777,216 points: 1024 ms
    of GPS L1 C/A at 16.384 MHz, the code repeated 1024 times, K = 1, 3
    Doppler bins) on the four-step kernels with single-column tiles (the
    4096 x 4096 split), against the FP64 oracle: Doppler bin exact, the peak
    exact modulo the 1 ms code period (the replica repeats), levels within
    the bar."""
    n, fs = 1 << 24, 16.384e6
    ca = unpack_codes(golden_codes, "gps_l1ca")
    em = signals.Emitter(ca[5], 1.023e6, 100.25, 0.5, 45.0, data_rate=0.0)
    raw = signals.synthesize([em], fs, n, 20.0, "ci16", seed=24)
    x = to_complex(raw)
    res, _ = run_engine(ctx, raw, fs, n, 1, [ca[5]], 1024, 0.5, 0.5)
    code = oracle.upsample(np.tile(ca[5], 1024), n)
    o64 = oracle.acquire(x, n, 1, code, fs, 0.5, 0.5, double=True)
    r, period = res[0], 16384
    assert r.doppler_bin == int(o64["doppler_bin"])
    assert r.index % period == int(o64["index"]) % period
    for f in ("level", "mean", "std", "snr", "sigma"):
        assert abs(getattr(r, f) - o64[f]) <= RTOL * abs(o64[f]), (f, getattr(r, f), o64[f])
