"""Device front end of the acquisition job (input_sampling_rate): the
Translate at the input rate and SequentialResampler run on the GPU before the
search, as AcquireGoldCodesL1 / AcquireL5 do on the host (fse.hpp:289-291,
312-314).  Checked against the oracle's mix -> resample -> acquire chain:
peak index and Doppler bin exact, magnitudes within 1e-4 of the FP64 oracle."""
import numpy as np
import pytest

from conftest import unpack_codes
from test_gpu_acquire import check_vs_oracle, run_engine, to_complex
from ugsdr_gb300 import signals

pytestmark = pytest.mark.gpu


def oracle_chain(oracle, raw, fs_in, fs, frontend):
    x = to_complex(raw)
    if frontend:
        x = oracle.table_mix(x, fs_in, frontend)
    return oracle.resample(x, int(fs), int(fs_in))


def test_gps_real_if_10mhz_to_4092khz(ctx, oracle, golden_codes):
    """Real int8 at 10 MHz, IF 2.5 MHz, resampled to 4.092 MHz (L = 1023, M = 2500)."""
    ca = unpack_codes(golden_codes, "gps_l1ca")
    ems = [signals.Emitter(ca[p], 1.023e6, ph, 2.5e6 + d, 50.0, 0.0) for p, ph, d in ((2, 100.25, 750.0), (9, 800.5, -1250.0))]
    raw = signals.synthesize(ems, 10e6, 20000, 20.0, "ri8", seed=11, real_if=True)
    fs_in, fs, if_hz = 10e6, 4.092e6, 2.5e6
    prns = [2, 9, 17]
    res, _ = run_engine(ctx, raw, fs, 4092, 2, [ca[p] for p in prns], 1, 2000, 500, input_sampling_rate=fs_in,
                        frontend_frequency=-if_hz, intermediate_frequency=if_hz, code_offset_ratio=fs_in / fs)
    y = oracle_chain(oracle, raw, fs_in, fs, -if_hz)
    for p, r in zip(prns, res):
        code = oracle.upsample(ca[p], 4092)
        kw = dict(if_freq=if_hz, ratio=fs_in / fs)
        check_vs_oracle(r, oracle.acquire(y, 4092, 2, code, fs, 2000, 500, **kw),
                        oracle.acquire(y, 4092, 2, code, fs, 2000, 500, double=True, **kw))
    assert abs(res[0].index - 100.25 / 1.023e6 * fs) <= 1.5
    assert abs(res[0].doppler - (2.5e6 + 750.0)) <= 250.0


def test_l5_real_if_40mhz_nh10_204600(ctx, oracle, golden_codes):
    """L5I at a 10 MHz real IF, 40 MHz int8, resampled to 20.46 MHz (L = 1023, M = 2000),
    10 ms coherent (N = 204,600) with the NH10 secondary code in the replica."""
    l5 = unpack_codes(golden_codes, "gps_l5i")
    sec = 1.0 - 2.0 * signals.NH10
    em = signals.Emitter(l5[6], 10.23e6, 61234.5, 10e6 - 400.0, 52.0, 0.0, secondary=sec)
    fs_in, fs = 40e6, 20.46e6
    raw = signals.synthesize([em], fs_in, 400000, 20.0, "ri8", seed=12, real_if=True)
    res, _ = run_engine(ctx, raw, fs, 204600, 1, [l5[6]], 10, 600, 200, sign_masks=[signals.nh10_mask()],
                        sign_segment=20460, input_sampling_rate=fs_in, frontend_frequency=-10e6,
                        intermediate_frequency=10e6, code_offset_ratio=fs_in / fs)
    y = oracle_chain(oracle, raw, fs_in, fs, -10e6)
    code = oracle.upsample(np.tile(l5[6], 10), 204600)
    for s in range(10):
        code[s * 20460:(s + 1) * 20460] *= sec[s]
    kw = dict(if_freq=10e6, ratio=fs_in / fs)
    check_vs_oracle(res[0], oracle.acquire(y, 204600, 1, code, fs, 600, 200, **kw),
                    oracle.acquire(y, 204600, 1, code, fs, 600, 200, double=True, **kw))
    assert abs(res[0].index - 61234.5 * 2) <= 2  # code phase within the NH period
    assert abs(res[0].doppler - (10e6 - 400.0)) <= 100.0


def test_ci16_pure_upsampling(ctx, oracle, golden_codes):
    """Ratio-1 resampling (2.046 -> 4.092 MHz, ZOH only) of int16 IQ with a front-end mix."""
    ca = unpack_codes(golden_codes, "gps_l1ca")
    em = signals.Emitter(ca[4], 1.023e6, 333.0, 150e3 + 500.0, 50.0, 0.0)
    raw = signals.synthesize([em], 2.046e6, 6138, 20.0, "ci16", seed=13)
    fs_in, fs = 2.046e6, 4.092e6
    res, _ = run_engine(ctx, raw, fs, 4092, 3, [ca[4]], 1, 1000, 500, input_sampling_rate=fs_in,
                        frontend_frequency=-150e3, intermediate_frequency=150e3, code_offset_ratio=0.5)
    y = oracle_chain(oracle, raw, fs_in, fs, -150e3)
    code = oracle.upsample(ca[4], 4092)
    kw = dict(if_freq=150e3, ratio=0.5)
    check_vs_oracle(res[0], oracle.acquire(y, 4092, 3, code, fs, 1000, 500, **kw),
                    oracle.acquire(y, 4092, 3, code, fs, 1000, 500, double=True, **kw))


def test_front_end_rejects(ctx, golden_codes):
    ca = unpack_codes(golden_codes, "gps_l1ca")
    raw = np.zeros(20000, np.int8)
    h = ctx.code_put(ca[1], 4092)
    try:
        for kw, msg in ((dict(input_sampling_rate=10e6 + 0.5), "integer"),
                        (dict(input_sampling_rate=10e6 + 1), "too large")):
            job = ctx.make_job(raw, 3, 4.092e6, 4092, 2, [h], 1000, 500, **kw)
            with pytest.raises(RuntimeError, match=msg):
                ctx.acquire(job)
        job = ctx.make_job(raw[:9000], 3, 4.092e6, 4092, 2, [h], 1000, 500, input_sampling_rate=10e6)
        with pytest.raises(RuntimeError, match="resampled"):
            ctx.acquire(job)
    finally:
        ctx.code_release(h)
