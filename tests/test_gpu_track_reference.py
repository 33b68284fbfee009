"""The tracking bank against the reference's own tracker.

tests/golden/track.npz holds the reference's TrackSingleSatellite run
(oracle/ref_track_harness.cpp: its TableMixer, UpdatePhase, CorrelateSplit,
Pll and Dll) on a seeded 4 MHz int8 capture: three GPS L1 C/A channels and
one Galileo E1B channel, 160 epochs, plus AddSignalImpl's refinement.

The bank runs in the reference's NCO mode (nco_mode 1: radian carrier phase,
a fresh 32-bit TableMixer NCO per epoch), E/P/L at 0.25 chip, PLL 25 Hz with
FLL 250 Hz, DLL 0.7 Hz - the reference's configuration.  Checks:
  * epoch 0 (the same starting state): E, P, L within 1e-4 of |P| of the
    reference's own taps;
  * every epoch, open loop: the bank's taps against the FP64 oracle's taps
    for the bank's own state at that epoch (the oracle's taps are pinned to
    the reference's within 1e-5, tests/test_oracle.py), within 1e-4 of the
    epoch's |P|; AddWithPhase (tracking_parameters.hpp:89-98) picks lhs +- rhs
    by a comparison that is a near-tie when one partial sum is tiny, so a tap
    may instead differ by twice that partial - each such tap is counted;
  * every epoch, the loop update: the oracle's Pll / Dll (pinned bit for bit
    to the reference's) fed the bank's taps gives the bank's states;
  * closed loop: the bank and the reference stay locked together (float
    sums in a different order make the trajectories drift apart slowly);
  * ugsdr_track_refine: the reference's offsets, acceptance and code phases.
The largest relative prompt error of each configuration is printed."""
import numpy as np
import pytest

from conftest import GOLDEN, unpack_codes
from ugsdr_gb300 import _lib as L

pytestmark = pytest.mark.gpu
RTOL = 1e-4
REF_CFG = dict(early_late=0.25, very_early_late=0.25, pll_bw=25.0, dll_bw=0.7, fll_bw=250.0)


def fixture():
    z = np.load(GOLDEN / "track.npz")
    raw = z["samples"]
    f = raw.astype(np.float32)
    x = (f[:, 0] + 1j * f[:, 1]).astype(np.complex64)
    fix = np.load(GOLDEN / "codes.npz")
    tables = {0: unpack_codes(fix, "gps_l1ca"), 6: unpack_codes(fix, "galileo_e1b")}
    chans = []
    for k in range(int(z["channels"])):
        pre = f"ch{k}/"
        sig = int(z[pre + "signal"])
        chans.append(dict(chips=tables[sig][int(z[pre + "prn"])], base=float(z[pre + "code_frequency"]),
                          code_phase=float(z[pre + "code_phase"]), carrier_frequency=float(z[pre + "carrier_frequency"]),
                          track=z[pre + "track"], refine_code_phase=float(z[pre + "refine_code_phase"]),
                          refine=z[pre + "refine"], boc=int(sig == 6)))
    return float(z["fs"]), raw, x, chans


def open_loop_errors(out, x, spm, fs, chips, base, ch0, el, vel, nco_mode, oracle):
    """Per epoch: max over the five taps of |tap - oracle tap| / |oracle P|,
    and the count of taps whose difference is explained only by an
    AddWithPhase near-tie (within twice the minor partial sum)."""
    period = int(round(len(chips) / base * 1000))
    n = len(out)
    taps = out["taps"].reshape(n, 10).astype(np.float64)
    worst, ties = np.zeros(n), 0
    for e in range(n):
        if e == 0:
            cf, cph, cp = ch0["carrier_frequency"], ch0.get("carrier_phase", 0.0), ch0["code_phase"]
        else:
            cf, cph, cp = out["carrier_frequency"][e - 1], out["carrier_phase"][e - 1], out["code_phase"][e - 1]
        ph = cp - fs / 1e3 * (e % period)
        o = oracle.track_taps(x[e * spm:(e + 1) * spm], chips, fs, base, ph, cf, cph, el, vel, nco_mode=nco_mode)
        p = abs(o[4] + 1j * o[5])
        d = np.abs((taps[e, 0::2] + 1j * taps[e, 1::2]) - (o[0:10:2] + 1j * o[1:10:2]))
        tie = d > RTOL * p
        assert (d[tie] <= 2.0 * o[10:15][tie] * 1.0001 + RTOL * p).all(), (e, d, o[10:15], p)
        ties += int(tie.sum())
        worst[e] = (d[~tie] / p).max() if (~tie).any() else 0.0
    return worst, ties


def test_reference_mode_bank_vs_reference_tracker(ctx, oracle):
    from ugsdr_gb300.api import TrackBank
    fs, raw, x, chans = fixture()
    spm = int(fs / 1000)
    n_ep = chans[0]["track"].shape[0]
    bank_chans = [dict(code=i, fs=fs, code_frequency=c["base"], code_phase=c["code_phase"],
                       carrier_frequency=c["carrier_frequency"], boc=c["boc"]) for i, c in enumerate(chans)]
    bank = TrackBank(ctx, bank_chans, [c["chips"] for c in chans], nco_mode=1, **REF_CFG)
    out = bank.run(raw, L.SAMPLES_CI8, n_ep)
    bank.close()
    for i, c in enumerate(chans):
        o, tr = out[:, i], c["track"]
        name = f"channel {i}"
        # epoch 0: the same state as the reference's first epoch
        ref0 = tr[0, 0:6:2] + 1j * tr[0, 1:6:2]
        got0 = o["taps"][0, 1:4, 0] + 1j * o["taps"][0, 1:4, 1]
        assert np.abs(got0 - ref0).max() <= RTOL * abs(ref0[1]), (name, got0, ref0)
        # open loop, every epoch
        worst, ties = open_loop_errors(o, x, spm, fs, c["chips"], c["base"], bank_chans[i], 0.25, 0.25, 1, oracle)
        print(f"reference mode, {name}: max |dP| / |P| {worst.max():.2e} over {n_ep} epochs, {ties} near-tie taps")
        assert worst.max() <= RTOL and ties <= 0.02 * 5 * n_ep, name
        # the loop update on the bank's own taps
        taps = np.stack([o["taps"][:, t, k] for t in (1, 2, 3) for k in (0, 1)], axis=1).astype(np.float64)
        loop = oracle.track_loop(taps, fs, c["base"], c["code_phase"], c["carrier_frequency"])
        assert np.abs(loop[:, 0] - o["carrier_frequency"]).max() <= 1e-4, name
        assert np.abs(loop[:, 1] - o["carrier_phase"]).max() <= 1e-6, name
        assert np.abs(loop[:, 2] - o["code_phase"]).max() <= 1e-5, name
        assert np.abs(loop[:, 3] - o["code_frequency"]).max() <= 1e-5, name
        # closed loop: locked together with the reference
        assert np.abs(o["carrier_frequency"] - tr[:, 6]).max() <= 1.0, name
        assert np.abs(o["code_phase"] - tr[:, 8]).max() <= 0.1, name
        p_ref = np.abs(tr[:, 2] + 1j * tr[:, 3])
        p_got = np.abs(o["taps"][:, 2, 0] + 1j * o["taps"][:, 2, 1])
        assert np.abs(p_got - p_ref).max() <= 0.05 * p_ref.max(), name


def test_refine_vs_reference(ctx):
    """ugsdr_track_refine from a code phase 3 samples off: the reference's
    offset, acceptance and refined code phase on all four channels (1 ms GPS
    codes and the 4 ms Galileo E1B code)."""
    from ugsdr_gb300.api import track_refine
    fs, raw, _, chans = fixture()
    ch = [dict(code=i, fs=fs, code_frequency=c["base"], code_phase=c["refine_code_phase"],
               carrier_frequency=c["carrier_frequency"]) for i, c in enumerate(chans)]
    acc, offs, refined = track_refine(ctx, ch, [c["chips"] for c in chans], raw, L.SAMPLES_CI8)
    for i, c in enumerate(chans):
        assert offs[i] == int(c["refine"][0]) and acc[i] == int(c["refine"][1]), (i, offs, acc, c["refine"])
        assert refined[i]["code_phase"] == c["refine"][2], i


def test_bank_at_256_channels_20mhz_open_loop(ctx, oracle):
    """The benchmark's tracking shape (256 channels GPS L1 C/A and Galileo
    E1B / E1C, int16 I/Q at 20 MHz, VE/E/P/L/VL at 0.5 / 0.15 chip, PLL 15 Hz,
    DLL 1 Hz, 64-bit carrier NCO) over 200 epochs: every epoch's taps of
    every channel against the FP64 oracle's for the bank's own state.  Bar:
    1e-4 of the epoch's |P| on the 36 signal channels; on the 220 channels
    with no signal |P| is noise that passes near zero, so there the bar is
    1e-4 of the channel's median |P|."""
    torch = pytest.importorskip("torch")
    import sys
    from concurrent.futures import ThreadPoolExecutor
    from conftest import ROOT
    sys.path.insert(0, str(ROOT))
    import bench
    from ugsdr_gb300.api import TrackBank
    n_ep = 200
    cap, chans, codes = bench.track_capture(0, n_ep / 1000)
    raw = cap.cpu().numpy()
    del cap
    torch.cuda.empty_cache()
    f = raw.astype(np.float32)
    x = (f[:, 0] + 1j * f[:, 1]).astype(np.complex64)
    bank = TrackBank(ctx, chans, codes, **bench.TRACK_CFG)
    out = bank.run(raw, L.SAMPLES_CI16, n_ep)
    bank.close()
    fs = chans[0]["fs"]
    spm = int(fs / 1000)
    el, vel = bench.TRACK_CFG["early_late"], bench.TRACK_CFG["very_early_late"]

    def one(i):
        c = chans[i]
        chips = codes[c["code"]]
        period = int(round(len(chips) / c["code_frequency"] * 1000))
        o = out[:, i]
        taps = o["taps"].reshape(n_ep, 10).astype(np.float64)
        errs, p_all, ties = np.zeros(n_ep), np.zeros(n_ep), 0
        for e in range(n_ep):
            if e == 0:
                cf, cph, cp = c["carrier_frequency"], 0.0, c["code_phase"]
            else:
                cf, cph, cp = o["carrier_frequency"][e - 1], o["carrier_phase"][e - 1], o["code_phase"][e - 1]
            r = oracle.track_taps(x[e * spm:(e + 1) * spm], chips, fs, c["code_frequency"], cp - fs / 1e3 * (e % period),
                                  cf, cph, el, vel)
            p = abs(r[4] + 1j * r[5])
            dp = abs((taps[e, 4] + 1j * taps[e, 5]) - (r[4] + 1j * r[5]))
            if RTOL * p < dp <= 2.0 * r[12] * 1.0001 + RTOL * p:  # AddWithPhase near-tie
                ties += 1
                dp = 0.0
            errs[e] = dp
            p_all[e] = p
        return errs, p_all, ties

    with ThreadPoolExecutor(max_workers=16) as ex:
        res = list(ex.map(one, range(len(chans))))
    worst_sig, worst_noise = 0.0, 0.0
    ties = sum(r[2] for r in res)
    for i, (errs, p_all, _) in enumerate(res):
        if i < 36:
            worst_sig = max(worst_sig, (errs / p_all).max())
        else:
            worst_noise = max(worst_noise, (errs / np.median(p_all)).max())
    print(f"256 channels, 20 MHz, {n_ep} epochs: max |dP| / |P| {worst_sig:.2e} (signal channels), "
          f"{worst_noise:.2e} of the median |P| (noise channels), {ties} near-tie prompts")
    assert worst_sig <= RTOL and worst_noise <= RTOL and ties <= 0.02 * n_ep * len(chans)
