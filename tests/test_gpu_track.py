"""Tracking correlator bank (ugsdr_track_*) against the FP64 oracle
restatement of the reference's tracking step (oracle/track_oracle.cpp).

Two levels, because the carrier wipe-off uses the reference's 6-bit phase
LUT: a phase difference of 1e-9 cycles between two runs eventually moves one
sample to the neighbouring LUT entry, so closed-loop trajectories that differ
only by FP32-versus-FP64 rounding drift apart by a few LUT steps.
  1. Correlator parity, open loop: every epoch's five taps recomputed by the
     oracle from the GPU's own NCO state at the start of that epoch must agree
     within 1e-4 of the channel's peak prompt magnitude (AddWithPhase's sign
     choice, a near-tie when one partial sum is tiny, may differ on at most 2 %
     of the taps, and then by twice that partial).
  2. Loop parity, closed loop: the GPU and oracle trajectories agree within
     0.1 Hz (carrier), 1e-3 samples (code phase) and 0.1 chip/s (code
     frequency), and the loops lock."""
import numpy as np
import pytest

from conftest import unpack_codes
from ugsdr_gb300 import _lib as L
from ugsdr_gb300 import signals

pytestmark = pytest.mark.gpu
RTOL = 1e-4


def to_complex(raw):
    f = raw.astype(np.float32)
    return (f[:, 0] + 1j * f[:, 1]).astype(np.complex64)


def check_open_loop(out, x, spm, chips, fs, base, ch0, el, vel, name):
    period = int(round(len(chips) / base * 1000))
    taps = out["taps"].reshape(len(out), 10).astype(np.float64)
    ref = np.zeros((len(out), 15))
    for e in range(len(out)):
        if e == 0:
            cf, cph, cp = ch0["carrier_frequency"], ch0.get("carrier_phase", 0.0), ch0["code_phase"]
        else:
            cf, cph, cp = out["carrier_frequency"][e - 1], out["carrier_phase"][e - 1], out["code_phase"][e - 1]
        ph = cp - fs / 1e3 * (e % period)
        ref[e] = __import__("pyoracle").track_taps(x[e * spm:(e + 1) * spm], chips, fs, base, ph, cf, cph, el, vel)
    scale = np.abs(ref[:, 4] + 1j * ref[:, 5]).max()
    diff = np.abs(taps - ref[:, :10]).reshape(len(out), 5, 2).max(axis=2)
    assert (diff <= RTOL * scale + 2.0 * ref[:, 10:15] * 1.0001).all(), name
    assert (diff > RTOL * scale).mean() <= 0.02, name


def check_closed_loop(out, ref, name):
    assert np.abs(out["carrier_frequency"] - ref[:, 10]).max() <= 0.1, name
    assert np.abs(out["code_phase"] - ref[:, 12]).max() <= 1e-3, name
    assert np.abs(out["code_frequency"] - ref[:, 13]).max() <= 0.1, name  # chips/s, 1e-7 of 1.023e6


def test_gps_l1_bank_vs_oracle(ctx, oracle, golden_codes):
    """Three GPS L1 C/A channels, int8 I/Q at 4 MHz, 120 epochs in two calls, reference loop constants."""
    from ugsdr_gb300.api import TrackBank
    ca = unpack_codes(golden_codes, "gps_l1ca")
    codes = {p: ca[p] for p in range(8)}
    raw, truth = signals.gps_l1_config(seed=21, codes=codes, fs=4e6, ms=120, visible=3, cn0=(45, 50), max_doppler=3000)
    x = to_complex(raw)
    chans, chips = [], []
    for i, t in enumerate(truth):
        chips.append(ca[t["prn"]])
        # acquisition hand-off: Doppler to the 50 Hz grid, code phase to the sample
        chans.append(dict(code=i, fs=4e6, code_frequency=1.023e6, code_phase=float(round(t["code_phase_samples"])),
                          carrier_frequency=round(t["doppler"] / 50) * 50.0))
    bank = TrackBank(ctx, chans, chips)
    out = np.concatenate([bank.run(raw[:60 * 4000], L.SAMPLES_CI8, 60), bank.run(raw[60 * 4000:], L.SAMPLES_CI8, 60)])
    bank.close()
    for i, (ch, t) in enumerate(zip(chans, truth)):
        name = f"prn {t['prn']}"
        check_open_loop(out[:, i], x, 4000, chips[i], 4e6, 1.023e6, ch, 0.25, 0.5, name)
        ref = oracle.track(x, 4000, 120, chips[i], 4e6, 1.023e6, ch["code_phase"], ch["carrier_frequency"])
        check_closed_loop(out[:, i], ref, name)
        # the loop locks: prompt dominates the early tap, frequency near the truth
        p = np.abs(out["taps"][60:, i, 2, 0] + 1j * out["taps"][60:, i, 2, 1]).mean()
        e = np.abs(out["taps"][60:, i, 1, 0] + 1j * out["taps"][60:, i, 1, 1]).mean()
        assert p > e, name
        assert abs(out["carrier_frequency"][-1, i] - t["doppler"]) < 30.0, name


def test_galileo_e1b_bank_vs_oracle(ctx, oracle, golden_codes):
    """BOC(1,1) E1B channel (4 ms code period), int16 I/Q at 10 MHz, VE/E/P/L/VL at 0.5/0.15 chip, PLL 15 Hz, DLL 1 Hz."""
    from ugsdr_gb300.api import TrackBank
    e1b = unpack_codes(golden_codes, "galileo_e1b")
    em = signals.Emitter(e1b[5], 2.046e6, 3000.0, 1200.0, 50.0, data_rate=250.0)
    raw = signals.synthesize([em], 10e6, 10000 * 40, 20.0, "ci16", seed=8)
    x = to_complex(raw)
    cp = 3000.0 / 2.046e6 * 10e6
    chans = [dict(code=0, fs=10e6, code_frequency=2.046e6, code_phase=float(round(cp)), carrier_frequency=1200.0, boc=1)]
    kw = dict(early_late=0.15, very_early_late=0.5, pll_bw=15.0, dll_bw=1.0, fll_bw=0.0)
    bank = TrackBank(ctx, chans, [e1b[5]], **kw)
    out = bank.run(raw, L.SAMPLES_CI16, 40)
    bank.close()
    check_open_loop(out[:, 0], x, 10000, e1b[5], 10e6, 2.046e6, chans[0], 0.15, 0.5, "e1b")
    ref = oracle.track(x, 10000, 40, e1b[5], 10e6, 2.046e6, chans[0]["code_phase"], 1200.0, **kw)
    check_closed_loop(out[:, 0], ref, "e1b")


def test_bank_rejects_bad_configs(ctx, golden_codes):
    from ugsdr_gb300.api import TrackBank
    ca = unpack_codes(golden_codes, "gps_l1ca")
    with pytest.raises(L.UgsdrError):  # fractional kHz sampling rate
        TrackBank(ctx, [dict(code=0, fs=4.0005e6, code_frequency=1.023e6, code_phase=0.0, carrier_frequency=0.0)], [ca[0]])
    with pytest.raises(L.UgsdrError):  # code index out of range
        TrackBank(ctx, [dict(code=3, fs=4e6, code_frequency=1.023e6, code_phase=0.0, carrier_frequency=0.0)], [ca[0]])


def test_refine_handoff_vs_oracle(ctx, oracle, golden_codes):
    """ugsdr_track_refine (AddSignalImpl's code-phase refinement): channels
    started 2-3 samples off find the offset and are accepted; one started half
    a millisecond off is rejected; offsets and acceptance equal the oracle's."""
    from ugsdr_gb300.api import track_refine
    ca = unpack_codes(golden_codes, "gps_l1ca")
    codes = {p: ca[p] for p in range(8)}
    raw, truth = signals.gps_l1_config(seed=31, codes=codes, fs=4e6, ms=6, visible=3, cn0=(46, 50), max_doppler=3000)
    x = to_complex(raw)
    chips, chans = [], []
    for i, t in enumerate(truth):
        chips.append(ca[t["prn"]])
        cp = float(round(t["code_phase_samples"]))
        chans.append(dict(code=i, fs=4e6, code_frequency=1.023e6, code_phase=(cp + (2.0, -3.0, 2000.0)[i]) % 4000,
                          carrier_frequency=round(t["doppler"] / 50) * 50.0))
    acc, offs, refined = track_refine(ctx, chans, chips, raw, L.SAMPLES_CI8)
    o_acc, o_offs, o_phases, _ = oracle.track_refine(x, chans, chips)
    assert acc == o_acc and offs == o_offs, (acc, offs, o_acc, o_offs)
    assert acc == [1, 1, 0]
    assert [r["code_phase"] for r in refined] == o_phases
    for i in range(2):
        true_cp = float(round(truth[i]["code_phase_samples"]))
        assert abs((refined[i]["code_phase"] - true_cp + 2000) % 4000 - 2000) <= 1


def test_host_run_in_overlapped_chunks_equals_device_run(ctx, golden_codes):
    """A host-buffer run longer than one copy chunk (1000 epochs) goes through
    two staging slots with the copies overlapping the runs; its outputs equal,
    bit for bit, one device-buffer run of the same epochs from the same
    start."""
    torch = pytest.importorskip("torch")
    from ugsdr_gb300.api import TrackBank
    ca = unpack_codes(golden_codes, "gps_l1ca")
    codes = {p: ca[p] for p in range(8)}
    n_ep = 2300
    raw, truth = signals.gps_l1_config(seed=22, codes=codes, fs=4e6, ms=n_ep, visible=2, cn0=(45, 50),
                                       max_doppler=3000, sample_type="ci16")
    chans = [dict(code=i, fs=4e6, code_frequency=1.023e6, code_phase=float(round(t["code_phase_samples"])),
                  carrier_frequency=round(t["doppler"] / 50) * 50.0) for i, t in enumerate(truth)]
    chips = [ca[t["prn"]] for t in truth]
    host_bank = TrackBank(ctx, chans, chips)
    host_out = host_bank.run(raw, L.SAMPLES_CI16, n_ep)
    host_bank.close()
    dev_bank = TrackBank(ctx, chans, chips)
    d_raw = torch.from_numpy(raw.copy()).cuda()
    d_out = torch.empty(host_out.nbytes, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    dev_bank.run_device(d_raw.data_ptr(), L.SAMPLES_CI16, n_ep, d_out.data_ptr())
    ctx.synchronize()
    dev_out = d_out.cpu().numpy().view(host_out.dtype).reshape(host_out.shape)
    dev_bank.close()
    assert host_out.tobytes() == dev_out.tobytes()
