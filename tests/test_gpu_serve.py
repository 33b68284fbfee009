"""Serving loop (ugsdr_server_*): every result is the same alone and in the
mix (continuous batching must not change results), jobs overlap on the
device, and the queue and memory-admission limits are enforced."""
import time

import numpy as np
import pytest

from conftest import unpack_codes
from ugsdr_gb300 import _lib as L
from ugsdr_gb300 import signals
from ugsdr_gb300.api import Server

pytestmark = pytest.mark.gpu


def make_jobs(ctx, golden_codes):
    """Uneven jobs: 2.046 / 4 / 10 / 50 MHz, 1-4 ms coherent, K 1-10, int8 and int16."""
    ca = unpack_codes(golden_codes, "gps_l1ca")
    specs = [(2.046e6, 1, 6, "ci16", 500.0), (4e6, 1, 10, "ci8", 500.0), (4e6, 2, 3, "ci16", 250.0),
             (10e6, 1, 4, "ci8", 500.0), (50e6, 1, 2, "ci16", 1000.0), (4e6, 4, 2, "ci8", 125.0)]
    jobs, keep = [], []
    for i, (fs, t_ms, k, st, step) in enumerate(specs):
        n = int(fs * t_ms / 1000)
        codes = {p: ca[p] for p in range(3 + i)}
        raw, _ = signals.gps_l1_config(seed=40 + i, codes=codes, fs=fs, ms=t_ms * k, visible=2, sample_type=st)
        hs = [ctx.code_put(codes[p], n, repeats=t_ms) for p in codes]
        stype = L.SAMPLES_CI8 if st == "ci8" else L.SAMPLES_CI16
        jobs.append(ctx.make_job(raw, stype, fs, n, k, hs, 3000.0, step))
        keep.append(hs)
    return jobs, keep


def test_results_same_alone_and_in_mix(ctx, golden_codes):
    jobs, handles = make_jobs(ctx, golden_codes)
    try:
        alone = [ctx.acquire(j) for j in jobs]
        srv = Server(ctx, max_inflight=4)
        tickets = [srv.submit(j) for j in jobs for _ in range(3)]  # each job three times, interleaved
        srv.drain()
        mixed = [srv.poll(t) for t in tickets]
        stats = srv.stats()
        srv.close()
        for i, res in enumerate(mixed):
            ref = alone[i // 3]
            assert len(res) == len(ref)
            for a, b in zip(ref, res):
                assert (a.index, a.doppler_bin) == (b.index, b.doppler_bin)
                assert abs(a.level - b.level) <= 1e-6 * a.level and abs(a.snr - b.snr) <= 1e-6 * a.snr
        assert stats["completed"] == len(tickets) and stats["failed"] == 0
        assert stats["max_inflight_seen"] >= 2  # jobs were on the device together
    finally:
        for hs in handles:
            for h in hs:
                ctx.code_release(h)


def test_queue_full_and_budget(ctx, golden_codes):
    jobs, handles = make_jobs(ctx, golden_codes)
    try:
        srv = Server(ctx, max_inflight=1, queue_capacity=2)
        codes = []
        with pytest.raises(L.UgsdrError) as e:
            for _ in range(50):
                codes.append(srv.submit(jobs[4]))
        assert e.value.status == L.E_QUEUE_FULL
        srv.drain()
        for t in codes:
            assert srv.poll(t) is not None
        srv.close()
        # a budget below one job's scratch: refused with E_NOMEM when nothing else runs
        small = Server(ctx, max_inflight=2, memory_budget=1 << 20)
        t = small.submit(jobs[4])
        small.drain()
        with pytest.raises(L.UgsdrError) as e:
            small.poll(t)
        assert e.value.status == L.E_NOMEM
        small.close()
    finally:
        for hs in handles:
            for h in hs:
                ctx.code_release(h)


@pytest.mark.parametrize("policy", [L.SERVE_FIFO, L.SERVE_RESPONSE_RATIO])
def test_admission_order(ctx, golden_codes, policy):
    """One slot: while a long search runs, a long and a short one queue.  FIFO
    admits them in arrival order; the response-ratio policy admits the short
    one first (its (wait + service) / service is larger)."""
    ca = unpack_codes(golden_codes, "gps_l1ca")
    raw, _ = signals.gps_l1_config(seed=77, codes={p: ca[p] for p in range(8)}, fs=50e6, ms=8, visible=2,
                                   sample_type="ci16")
    long_h = [ctx.code_put(ca[p], 50000) for p in range(24)]
    short_h = [ctx.code_put(ca[0], 50000)]
    try:
        long_job = ctx.make_job(raw, L.SAMPLES_CI16, 50e6, 50000, 8, long_h, 5000.0, 250.0)
        short_job = ctx.make_job(raw, L.SAMPLES_CI16, 50e6, 50000, 1, short_h, 500.0, 500.0)
        srv = Server(ctx, max_inflight=1, policy=policy)
        first = srv.submit(long_job)
        time.sleep(0.002)
        t_long = srv.submit(long_job)
        t_short = srv.submit(short_job)
        done = {}
        t0 = time.perf_counter()
        while len(done) < 3 and time.perf_counter() - t0 < 120:
            for t in (first, t_long, t_short):
                if t not in done and srv.poll(t) is not None:
                    done[t] = time.perf_counter()
            time.sleep(0.0005)
        srv.close()
        assert len(done) == 3
        if policy == L.SERVE_FIFO:
            assert done[t_long] < done[t_short]
        else:
            assert done[t_short] < done[t_long]
    finally:
        for h in long_h + short_h:
            ctx.code_release(h)


def test_tracking_requests_same_alone_and_in_mix(ctx, golden_codes):
    """Tracking requests through the server (ugsdr_server_submit_track): a
    bank advanced by three consecutive requests (its channels' state kept on
    the device between them), interleaved with acquisition jobs on the other
    slots, produces the same outputs, bit for bit, as the same bank run in
    one call alone (Tracker::Track's epoch loop, tracker.hpp:186-197)."""
    from ugsdr_gb300.api import TrackBank
    ca = unpack_codes(golden_codes, "gps_l1ca")
    codes = {p: ca[p] for p in range(8)}
    n_ep = 90
    raw, truth = signals.gps_l1_config(seed=23, codes=codes, fs=4e6, ms=n_ep, visible=3, cn0=(44, 50), max_doppler=3000,
                                       sample_type="ci16")
    chans = [dict(code=i, fs=4e6, code_frequency=1.023e6, code_phase=float(round(t["code_phase_samples"])),
                  carrier_frequency=round(t["doppler"] / 50) * 50.0) for i, t in enumerate(truth)]
    chips = [ca[t["prn"]] for t in truth]
    alone_bank = TrackBank(ctx, chans, chips)
    alone = alone_bank.run(raw, L.SAMPLES_CI16, n_ep)
    alone_bank.close()
    jobs, handles = make_jobs(ctx, golden_codes)
    try:
        acq_alone = [ctx.acquire(j) for j in jobs]
        bank = TrackBank(ctx, chans, chips)
        srv = Server(ctx, max_inflight=4)
        tickets = []
        for s in range(3):
            tickets.append(("acq", s, srv.submit(jobs[s])))
            tickets.append(("trk", s, srv.submit_track(bank, raw[s * 30 * 4000:(s + 1) * 30 * 4000], L.SAMPLES_CI16, 30)))
            tickets.append(("acq", s + 3, srv.submit(jobs[s + 3])))
        srv.drain()
        parts = {}
        for kind, idx, t in tickets:
            out = srv.poll(t)
            assert out is not None
            if kind == "trk":
                parts[idx] = out
            else:
                for a, b in zip(acq_alone[idx], out):
                    assert (a.index, a.doppler_bin, a.level) == (b.index, b.doppler_bin, b.level)
        served = np.concatenate([parts[0], parts[1], parts[2]])
        assert served.tobytes() == alone.tobytes()
        assert srv.stats()["completed"] == 9
        srv.close()
        bank.close()
    finally:
        for hs in handles:
            for h in hs:
                ctx.code_release(h)
