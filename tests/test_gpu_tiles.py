"""Four-step tile shapes (ugsdr_tile_get / ugsdr_tile_set) and the autotuner
(ugsdr_autotune).

Every shape the autotuner may pick runs the same search: peak index and
Doppler bin equal to the oracle's, level, mean, sigma and SNR within 1e-4
of the FP64 oracle, on the compile-time 200 x 250 split of a 50,000-point
block (warp-owned and natural column kernels, 8 / 4 / 2 columns, 8 / 4 / 2
rows, warp-owned row kernels with staged or L2 code rows and CTA-tile row
kernels) and on the runtime splits of a 16,000-point block (125 x 128, its
transpose, 100 x 160), whose code spectra were cached under another split
and are rebuilt by the change.  The tuner keeps a shape it measured and
the search still matches the oracle after tuning."""
import numpy as np
import pytest

from conftest import unpack_codes
from test_gpu_acquire import RTOL, check_vs_oracle, to_complex
from ugsdr_gb300 import _lib as L
from ugsdr_gb300 import signals

pytestmark = pytest.mark.gpu

SHAPES_50K = ([dict(cols=c, rows=r, warp_cols=w, warp_rows=0) for w in (1, 0) for c in (8, 4, 2) for r in (8, 4, 2)] +
              [dict(cols=c, rows=r, warp_cols=1, warp_rows=w) for w in (1, 2) for c in (8, 2) for r in (8, 2)])
KEY = ("n1", "cols", "rows", "warp_cols", "warp_rows")


def gps_50k(golden_codes):
    ca = unpack_codes(golden_codes, "gps_l1ca")
    codes = {i: ca[i] for i in range(4)}
    raw, truth = signals.gps_l1_config(seed=9, codes=codes, fs=50e6, ms=2, visible=2, sample_type="ci16", cn0=(48, 50),
                                       max_doppler=1000)
    return ca, raw, [t["prn"] for t in truth]


def test_every_tuner_shape_of_50000_matches_oracle(ctx, oracle, golden_codes):
    ca, raw, prns = gps_50k(golden_codes)
    x = to_complex(raw)
    refs = []
    for p in prns:
        code = oracle.upsample(ca[p], 50000)
        refs.append((oracle.acquire(x, 50000, 2, code, 50e6, 1000, 500),
                     oracle.acquire(x, 50000, 2, code, 50e6, 1000, 500, double=True)))
    handles = [ctx.code_put(ca[p], 50000) for p in prns]
    try:
        rule = ctx.tile_shape(50000)
        assert (rule["n1"], rule["warp_cols"], rule["warp_rows"]) == (200, 1, 1)
        job = ctx.make_job(raw, L.SAMPLES_CI16, 50e6, 50000, 2, handles, 1000, 500)
        for shape in SHAPES_50K:
            ctx.set_tile_shape(50000, shape)
            got = ctx.tile_shape(50000)
            assert (got["cols"], got["rows"], got["warp_cols"], got["warp_rows"], got["n1"]) == \
                (shape["cols"], shape["rows"], shape["warp_cols"], shape["warp_rows"], 200), (shape, got)
            res, _ = ctx.acquire(job, cells=True)
            for r, (o32, o64) in zip(res, refs):
                check_vs_oracle(r, o32, o64)
    finally:
        ctx.set_tile_shape(50000, None)
        for h in handles:
            ctx.code_release(h)
    assert ctx.tile_shape(50000) == rule


@pytest.mark.parametrize("n1,cols,rows", [(0, 0, 0), (128, 0, 0), (100, 0, 0), (100, 2, 2), (128, 4, 8)])
def test_runtime_splits_of_16000_match_oracle(ctx, oracle, golden_codes, n1, cols, rows):
    """4 MHz, 4 ms blocks (16,000 = 125 x 128 by the rule): the code spectrum
    is cached under the rule's split before the shape changes."""
    chips = unpack_codes(golden_codes, "galileo_e1b")[7]
    em = signals.Emitter(chips, 2.046e6, 1234.25, 250.0, 60.0, data_rate=0.0)
    raw = signals.synthesize([em], 4e6, 32000, 20.0, "ci16", seed=23)
    x = to_complex(raw)
    code = oracle.upsample(chips, 16000)
    o32 = oracle.acquire(x, 16000, 2, code, 4e6, 500, 250)
    o64 = oracle.acquire(x, 16000, 2, code, 4e6, 500, 250, double=True)
    h = ctx.code_put(chips, 16000)
    try:
        assert ctx.tile_shape(16000)["n1"] == 125
        ctx.set_tile_shape(16000, dict(n1=n1, cols=cols, rows=rows))
        got = ctx.tile_shape(16000)
        assert got["n1"] == (n1 or 125) and (cols == 0 or got["cols"] == cols) and (rows == 0 or got["rows"] == rows)
        res, _ = ctx.acquire(ctx.make_job(raw, L.SAMPLES_CI16, 4e6, 16000, 2, [h], 500, 250), cells=True)
        check_vs_oracle(res[0], o32, o64)
    finally:
        ctx.set_tile_shape(16000, None)
        ctx.code_release(h)


def test_invalid_shapes_leave_the_old_one(ctx):
    before = ctx.tile_shape(50000)
    for bad, status in ((dict(n1=7), L.E_UNSUPPORTED),      # 7 does not divide 50,000
                        (dict(n1=2), L.E_UNSUPPORTED),        # 25,000-point rows exceed shared memory
                        (dict(cols=3), L.E_INVALID),         # not a power of two
                        (dict(rows=16), L.E_INVALID),
                        (dict(warp_cols=2), L.E_INVALID)):
        with pytest.raises(L.UgsdrError) as e:
            ctx.set_tile_shape(50000, bad)
        assert e.value.status == status, bad
        assert ctx.tile_shape(50000) == before
    with pytest.raises(L.UgsdrError) as e:  # single-CTA block size: no four-step tiles
        ctx.tile_shape(4000)
    assert e.value.status == L.E_INVALID


def test_autotune_keeps_a_measured_shape(ctx, oracle, golden_codes):
    ca, raw, prns = gps_50k(golden_codes)
    x = to_complex(raw)
    chips = unpack_codes(golden_codes, "galileo_e1b")[7]
    em = signals.Emitter(chips, 2.046e6, 1234.25, 250.0, 60.0, data_rate=0.0)
    raw16 = signals.synthesize([em], 4e6, 32000, 20.0, "ci16", seed=23)
    h50 = [ctx.code_put(ca[p], 50000) for p in prns]
    h16 = ctx.code_put(chips, 16000)
    try:
        jobs = [ctx.make_job(raw, L.SAMPLES_CI16, 50e6, 50000, 2, h50, 1000, 500),
                ctx.make_job(raw16, L.SAMPLES_CI16, 4e6, 16000, 2, [h16], 500, 250)]
        tried = ctx.autotune(jobs)
        for n in (50000, 16000):
            mine = [t for t in tried if t["block_samples"] == n]
            assert len(mine) >= 4 and all(t["ms"] > 0 for t in mine), mine
            kept = ctx.tile_shape(n)
            key = lambda t: tuple(t[k] for k in KEY)
            assert key(kept) in {key(t) for t in mine}
            best = min(t["ms"] for t in mine)
            kept_ms = [t["ms"] for t in mine if key(t) == key(kept)][0]
            if key(kept) != key(mine[0]):  # mine[0]: the rule's shape, measured first
                assert kept_ms == best and kept_ms < 0.97 * mine[0]["ms"]
            print(f"N={n}: kept {kept} of {len(mine)} shapes ({kept_ms:.3f} ms; rule {mine[0]['ms']:.3f} ms)")
        res, _ = ctx.acquire(jobs[0], cells=True)
        for p, r in zip(prns, res):
            code = oracle.upsample(ca[p], 50000)
            check_vs_oracle(r, oracle.acquire(x, 50000, 2, code, 50e6, 1000, 500),
                            oracle.acquire(x, 50000, 2, code, 50e6, 1000, 500, double=True))
        res, _ = ctx.acquire(jobs[1], cells=True)
        code = oracle.upsample(chips, 16000)
        x16 = to_complex(raw16)
        check_vs_oracle(res[0], oracle.acquire(x16, 16000, 2, code, 4e6, 500, 250),
                        oracle.acquire(x16, 16000, 2, code, 4e6, 500, 250, double=True))
    finally:
        ctx.set_tile_shape(50000, None)
        ctx.set_tile_shape(16000, None)
        for h in h50 + [h16]:
            ctx.code_release(h)
