"""CudaFastSearchEngine (include/ugsdr_cuda_engine.hpp): the reference's
FastSearchEngineBase::Process call shape (src/acquisition/fse.hpp:450-507)
in C++ over ugsdr_acquire_batch, built without the reference's headers.

CPU: the header compiles, the program links against libugsdr_cuda.so, and
its AdjustSamplingRate is fse.hpp:222-240's.  GPU: the program runs on the
reference's real_8 capture (the first 4 ms, as the reference's FSE reads,
test/integration_tests.cpp:406-409): its kept satellites are the known
answer's (253-263; 8 of 8 within 400 Hz, the reference asks 4), and each
equals ugsdr_acquire's result for the same search (AcquireGoldCodesL1's job:
+9.55 MHz translate, AdjustSamplingRate to 9.548 MHz, 4 ms codes folded to
1 ms after |.|)."""
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, unpack_codes
from ugsdr_gb300 import _lib as L

BIN = ROOT / "tests" / "native" / "_bin" / "cuda_engine_run"
L1 = 1575.42e6


def build(lib):
    BIN.parent.mkdir(exist_ok=True)
    libdir = ROOT / "ugsdr_gb300" / "_lib"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "native" / "cuda_engine_run.cpp"), "-L", str(libdir), "-lugsdr_cuda",
           f"-Wl,-rpath,{libdir}", "-o", str(BIN)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_engine_compiles_and_links(lib):
    build(lib)
    assert BIN.exists()


def test_adjust_sampling_rate_matches_reference(lib):
    """The engine's AdjustSamplingRate against fse.hpp:222-240 restated here:
    the whole-kHz divisor closest to the target, or the input rate when the
    candidates run out."""
    build(lib)

    def adjust(fs, target):
        new = fs
        for i in range(1, int(2 * fs / target)):
            cand = fs / i
            if (cand / 1e3) % 1 != 0.0:
                continue
            if abs(target - cand) > abs(target - new):
                return new
            new = cand
        return fs
    cases = [(38.192e6, 8.192e6, 9.548e6), (38.192e6, 2.048e6, 1.736e6), (38.192e6, 40.96e6, 38.192e6),
             (50e6, 8.192e6, 10e6), (4e6, 8.192e6, 4e6), (40e6, 20.46e6, 40e6), (33.25e6, 8.192e6, None)]
    for fs, target, want in cases:
        r = subprocess.run([str(BIN), "--rate", repr(fs), repr(target)], capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stderr
        got = float(r.stdout)
        assert got == adjust(fs, target), (fs, target, got)
        if want is not None:
            assert got == want, (fs, target, got)


@pytest.mark.gpu
def test_engine_real_8_known_answer(lib, ctx):
    build(lib)
    z = np.load(GOLDEN / "real8.npz")
    raw = z["samples"]
    fs, f_if = float(z["fs"]), float(z["if_hz"])
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "real8.bin"
        raw.tofile(path)
        r = subprocess.run([str(BIN), str(path), str(L.SAMPLES_RI8), repr(fs), repr(L1 + f_if), "6000", "200"],
                           capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = [l.split() for l in r.stdout.splitlines() if l.strip()]
    got = {int(x[1]): dict(doppler=float(x[3]), code_offset=float(x[4]), level=float(x[5]), sigma=float(x[6]),
                           f_if=float(x[7])) for x in rows if int(x[0]) == 0}
    found = [int(sv) for sv, dop, _ in z["kat"]
             if int(sv) in got and abs(got[int(sv)]["doppler"] - got[int(sv)]["f_if"] - dop) <= 400]
    assert len(found) == 8, (found, got)
    # the same search through ugsdr_acquire
    new_fs = 9.548e6
    n = int(round(new_fs * 4 / 1000))
    ca = unpack_codes(np.load(GOLDEN / "codes.npz"), "gps_l1ca")
    handles = [ctx.code_put(ca[sv], n, repeats=4) for sv in range(32)]
    try:
        job = ctx.make_job(raw[: int(fs * 4 / 1000)], L.SAMPLES_RI8, new_fs, n, 1, handles, 6000, 200,
                           input_sampling_rate=fs, frontend_frequency=f_if, intermediate_frequency=-f_if,
                           code_offset_ratio=fs / new_fs, fold_samples=n // 4, fold_coherent=True)
        res = ctx.acquire(job)
    finally:
        for h in handles:
            ctx.code_release(h)
    kept = {sv for sv in range(32) if res[sv].snr > 3.3}
    assert kept == set(got)
    for sv in kept:
        assert got[sv]["doppler"] == pytest.approx(res[sv].doppler, abs=1e-6)
        assert got[sv]["code_offset"] == pytest.approx(res[sv].code_offset, abs=1e-6)
        assert got[sv]["level"] == pytest.approx(res[sv].level, rel=1e-6)
