"""Observables from tracking outputs (ugsdr_preamble_search, ugsdr_observables)
against the reference and the oracle restatement of src/measurements/
observable.hpp.

  * Preamble candidates: the fixture lists come from the reference's own
    matched filter (tests/golden/preamble.npz); the device lists must equal
    them exactly, for GPS LNAV and GLONASS, odd lengths, prompts shorter than
    the preamble, an inverted stream and an all-zero prompt.
  * Observable arithmetic against the reference's own Observable
    (tests/golden/observables.npz: its constructor, CalculateSnr and
    UpdatePseudoranges on the reference tracker's histories): pseudorange and
    Doppler bit for bit, pseudophase within 1e-9 cycles, SNR within 1e-5 dB.
  * Observable arithmetic on a real tracking run against the oracle:
    pseudorange and Doppler bit for bit (the same double operations), SNR
    within a float ulp of 27 dB (log10f), pseudophase within 1e-5 cycles (the
    bank keeps the carrier phase as a 64-bit fraction of a cycle, the
    reference accumulates radians in double)."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from conftest import unpack_codes
from ugsdr_gb300 import _lib as L
from ugsdr_gb300 import signals

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).parent / "golden" / "preamble.npz"
CASES = ("gps_two_subframes", "gps_inverted", "gps_odd_length", "gps_shorter_than_preamble", "gps_zeros",
         "glonass_strings", "glonass_odd_length", "glonass_shorter_than_preamble")


def bank_rows(prompt_i: np.ndarray) -> np.ndarray:
    """(n_epochs, n_channels) tracking outputs carrying the given prompt I."""
    from ugsdr_gb300.api import TRACK_DTYPE
    rows = np.zeros(prompt_i.shape, TRACK_DTYPE)
    rows["taps"][:, :, 2, 0] = prompt_i
    rows["taps"][:, :, 2, 1] = 1.0
    return rows


@pytest.mark.parametrize("case", CASES)
def test_preamble_search_matches_reference(ctx, case):
    from ugsdr_gb300.api import preamble_search
    z = np.load(GOLDEN)
    x = z[f"{case}/prompt_i"].astype(np.float32)
    got = preamble_search(ctx, bank_rows(x[:, None]), [int(z[f"{case}/message"])], cap=len(x))
    assert got == [z[f"{case}/indexes"].tolist()]


def test_preamble_search_many_channels_and_cap(ctx, oracle):
    """Six channels of 12,000 epochs in one call, GPS and GLONASS mixed, equal
    to the oracle per channel; a cap below the count keeps the first ones and
    still reports the count."""
    from ugsdr_gb300.api import preamble_search
    z = np.load(GOLDEN)
    rng = np.random.default_rng(9)
    cols = [z["gps_two_subframes/prompt_i"], z["gps_inverted/prompt_i"], np.zeros(12000, np.int8)]
    glo = np.repeat(rng.choice([-1, 1], 1200), 10) * 30 + rng.normal(0, 10, 12000)
    cols += [np.clip(glo, -127, 127).astype(np.int8), rng.integers(-5, 6, 12000).astype(np.int8),
             z["gps_two_subframes/prompt_i"][::-1].copy()]
    msgs = [0, 0, 0, 1, 1, 0]
    x = np.stack(cols, axis=1).astype(np.float32)
    got = preamble_search(ctx, bank_rows(x), msgs, cap=12000)
    for c in range(x.shape[1]):
        assert got[c] == oracle.preamble_search(x[:, c], msgs[c], cap=12000), c
    counts = (C.c_int * 6)()
    idx = np.zeros((6, 5), np.int32)
    rows = bank_rows(x)
    st = ctx.lib.ugsdr_preamble_search(ctx.h, rows.ctypes.data, 0, 12000, 6, (C.c_int * 6)(*msgs), counts,
                                       idx.ctypes.data_as(C.POINTER(C.c_int)), 5)
    assert st == L.OK
    assert list(counts) == [len(g) for g in got]
    for c in range(6):
        assert idx[c, :min(5, counts[c])].tolist() == got[c][:5]


def test_preamble_search_rejects_bad_input(ctx):
    from ugsdr_gb300.api import preamble_search
    rows = bank_rows(np.ones((100, 1), np.float32))
    with pytest.raises(L.UgsdrError):
        preamble_search(ctx, rows, [7])


def gps_run(ctx, golden_codes, n_ep, seed=31):
    from ugsdr_gb300.api import TrackBank
    ca = unpack_codes(golden_codes, "gps_l1ca")
    codes = {p: ca[p] for p in range(8)}
    raw, truth = signals.gps_l1_config(seed=seed, codes=codes, fs=4e6, ms=n_ep, visible=3, cn0=(44, 50),
                                       max_doppler=3000)
    chans = [dict(code=i, fs=4e6, code_frequency=1.023e6, code_phase=float(round(t["code_phase_samples"])),
                  carrier_frequency=round(t["doppler"] / 50) * 50.0, carrier_phase=0.5 * i)
             for i, t in enumerate(truth)]
    bank = TrackBank(ctx, chans, [ca[t["prn"]] for t in truth])
    return bank, raw, chans


def obs_channels(chans, if_hz):
    return [dict(fs=ch["fs"], intermediate_frequency=if_hz, carrier_frequency=ch["carrier_frequency"],
                 carrier_phase=ch["carrier_phase"], preamble_position=17 + 5 * i, range_correction_ms=68.0 + i)
            for i, ch in enumerate(chans)]


def test_observables_match_reference(ctx):
    """ugsdr_observables on the reference tracker's own outputs (three GPS
    channels, 160 epochs) against the reference Observable's outputs."""
    from conftest import reference_track_rows
    from ugsdr_gb300.api import TRACK_DTYPE, observables
    z = np.load(GOLDEN.parent / "observables.npz")
    ref_rows, cf0, fs = reference_track_rows(range(int(z["channels"])))
    rows = np.zeros(ref_rows.shape, TRACK_DTYPE)
    for name in TRACK_DTYPE.names:
        rows[name] = ref_rows[name]
    och = [dict(fs=fs, intermediate_frequency=float(z["intermediate_frequency"]), carrier_frequency=cf,
                carrier_phase=0.0, preamble_position=int(z["position"]), range_correction_ms=68.0) for cf in cf0]
    got = observables(ctx, rows, och)
    for c in range(rows.shape[1]):
        ref = z[f"ch{c}"]
        np.testing.assert_array_equal(got["pseudorange"][:, c], ref[:, 0])
        np.testing.assert_array_equal(got["doppler"][:, c], ref[:, 2])
        np.testing.assert_allclose(got["pseudophase"][:, c], ref[:, 1], rtol=0, atol=1e-9)
        np.testing.assert_allclose(got["snr"][:, c], ref[:, 3], rtol=0, atol=1e-5)
        print(f"channel {c}: max |d pseudophase| {np.abs(got['pseudophase'][:, c] - ref[:, 1]).max():.1e} cycles, "
              f"max |d snr| {np.abs(got['snr'][:, c] - ref[:, 3]).max():.1e} dB")


def test_observables_match_oracle(ctx, oracle, golden_codes):
    """Three GPS channels tracked over 2,100 epochs (three scan segments),
    then their observables against the oracle on the same tracking rows."""
    from ugsdr_gb300.api import observables
    bank, raw, chans = gps_run(ctx, golden_codes, 2100)
    rows = bank.run(raw, L.SAMPLES_CI8, 2100)
    bank.close()
    # a nonzero IF exercises the windup and Doppler terms on the same rows
    for if_hz in (0.0, 1.25e3):
        och = obs_channels(chans, if_hz)
        got = observables(ctx, rows, och)
        for c, ch in enumerate(och):
            ref = oracle.observables(rows[:, c], ch["fs"], if_hz, ch["carrier_frequency"], ch["carrier_phase"],
                                     ch["preamble_position"], ch["range_correction_ms"])
            np.testing.assert_array_equal(got["pseudorange"][:, c], ref[:, 0])
            np.testing.assert_array_equal(got["doppler"][:, c], ref[:, 2])
            np.testing.assert_allclose(got["pseudophase"][:, c], ref[:, 1], rtol=0, atol=1e-5)
            np.testing.assert_allclose(got["snr"][:, c], ref[:, 3], rtol=0, atol=1e-5)


def test_observables_device_chain_equals_host(ctx, golden_codes):
    """Tracking and observables on device buffers (ugsdr_track_run_device,
    then ugsdr_observables on its outputs) give the host call's results."""
    torch = pytest.importorskip("torch")
    from ugsdr_gb300.api import OBSERVABLE_DTYPE, observables, preamble_search
    bank, raw, chans = gps_run(ctx, golden_codes, 1200, seed=32)
    host_rows = bank.run(raw, L.SAMPLES_CI8, 1200)
    bank.close()
    och = obs_channels(chans, 0.0)
    host = observables(ctx, host_rows, och)
    bank2, _, _ = gps_run(ctx, golden_codes, 1200, seed=32)
    d_raw = torch.from_numpy(raw.copy()).cuda()
    d_rows = torch.empty(host_rows.nbytes, dtype=torch.uint8, device="cuda")
    d_obs = torch.empty(host.nbytes, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    bank2.run_device(d_raw.data_ptr(), L.SAMPLES_CI8, 1200, d_rows.data_ptr())
    ctx.synchronize()
    bank2.close()
    observables(ctx, d_rows.data_ptr(), och, shape=host_rows.shape, out_ptr=d_obs.data_ptr())
    dev = d_obs.cpu().numpy().view(OBSERVABLE_DTYPE).reshape(host.shape)
    assert dev.tobytes() == host.tobytes()
    msgs = [0] * len(chans)
    assert preamble_search(ctx, d_rows.data_ptr(), msgs, shape=host_rows.shape) == preamble_search(ctx, host_rows, msgs)


def test_observables_reject_bad_channels(ctx):
    from ugsdr_gb300.api import observables
    rows = bank_rows(np.ones((50, 1), np.float32))
    with pytest.raises(L.UgsdrError):
        observables(ctx, rows, [dict(fs=4e6, carrier_frequency=0.0, preamble_position=50)])
    with pytest.raises(L.UgsdrError):
        observables(ctx, rows, [dict(fs=0.0, carrier_frequency=0.0)])
