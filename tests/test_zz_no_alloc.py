"""The allocation-free entry point ugsdr_acquire_static.

Callers that cannot allocate device memory themselves (real-time receiver
loops that must not block on cudaMalloc, and host applications whose device
memory belongs to another allocator or pool) pass device pointers for inputs
and outputs; the library's scratch is a fixed-size file-scope device array.
These tests call it through the C ABI twice in a row per case and check its
cells against ugsdr_acquire's on the same input (index exact, level/mean/std
within 1e-4 relative), over the sample types, both spectrum modes, both fold
modes and a front-end translate, all on a non-blocking stream (the first call
on a device also uploads the mixer table, which must be ordered before that
call's kernels whatever stream the caller uses); and that a job beyond the
scratch limit is rejected.  The file sits where pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

from conftest import unpack_codes
from ugsdr_gb300 import _lib as L

pytestmark = pytest.mark.gpu
RTOL = 1e-4
FS = 4e6
N = 4000
CELL = np.dtype([("level", "<f4"), ("index", "<u4"), ("mean", "<f4"), ("std", "<f4")])


def _samples(raw_ci8: np.ndarray, sample_type: int) -> np.ndarray:
    if sample_type == L.SAMPLES_CI8:
        return raw_ci8.copy()
    if sample_type == L.SAMPLES_CI16:
        return (raw_ci8.astype(np.int16) * 37).astype(np.int16)
    if sample_type == L.SAMPLES_CF32:
        return (raw_ci8.astype(np.float32) * 0.25).astype(np.float32)
    return raw_ci8[:, 0].copy()  # real int8 IF: the I channel


# (name, sample type, K, fold samples, fold coherent, spectrum mode, front-end frequency)
CASES = [
    ("ci8-plain", L.SAMPLES_CI8, 10, 0, 1, L.SPECTRUM_ONE_SIDED, 0.0),
    ("cf32", L.SAMPLES_CF32, 3, 0, 1, L.SPECTRUM_ONE_SIDED, 0.0),
    ("ci16-two-sided", L.SAMPLES_CI16, 3, 0, 1, L.SPECTRUM_TWO_SIDED, 0.0),
    ("ri8-frontend", L.SAMPLES_RI8, 2, 0, 1, L.SPECTRUM_ONE_SIDED, 1.25e6),
    ("ci8-fold-coherent", L.SAMPLES_CI8, 3, 1000, 1, L.SPECTRUM_ONE_SIDED, 0.0),
    ("ci16-fold-noncoherent", L.SAMPLES_CI16, 3, 1000, 0, L.SPECTRUM_TWO_SIDED, 750.0),
]


@pytest.mark.parametrize("name,stype,k,fold,coherent,mode,fe", CASES, ids=[c[0] for c in CASES])
def test_static_entry_matches_acquire(ctx, acq_golden, golden_codes, name, stype, k, fold, coherent, mode, fe):
    torch = pytest.importorskip("torch")
    lib = L.load()
    ca = unpack_codes(golden_codes, "gps_l1ca")
    samples = _samples(acq_golden["acq_raw"], stype)
    n_samples = samples.shape[0]
    prns = [int(p) for p in acq_golden["acq_prns"]][:3]
    rng, step = (5000.0, 500.0) if k == 10 else (2000.0, 500.0)
    from ugsdr_gb300 import api
    code_samples = np.stack([api.repeat_upsample(ca[p], 1, N) for p in prns]).astype(np.float32)

    # the entry point with context allocations, on the same job
    hs = [ctx.code_put(ca[p], N, spectrum_mode=mode) for p in prns]
    try:
        job_ref = ctx.make_job(samples, stype, FS, N, k, hs, rng, step, n_samples=n_samples, frontend_frequency=fe,
                               fold_samples=fold, fold_coherent=bool(coherent), spectrum_mode=mode)
        _, ref_cells = ctx.acquire(job_ref, cells=True)
    finally:
        for h in hs:
            ctx.code_release(h)

    dev = torch.device("cuda", 0)
    d_samples = torch.from_numpy(samples).to(dev)
    d_codes = torch.from_numpy(code_samples).to(dev)
    n_dop = ref_cells.shape[1]
    d_cells = torch.zeros(len(prns) * n_dop * 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)  # torch streams are non-blocking
    job = L.StaticJob(d_samples.data_ptr(), stype, n_samples, FS, fe, N, k, fold, coherent, rng, step,
                      d_codes.data_ptr(), len(prns), L.STAT_ABS, mode)
    torch.cuda.synchronize()
    for call in range(2):
        with torch.cuda.stream(stream):
            d_cells.fill_(-1.0)
        need = C.c_size_t()
        st = lib.ugsdr_acquire_static(C.c_void_p(stream.cuda_stream), C.byref(job), C.c_void_p(d_cells.data_ptr()),
                                      C.byref(need))
        assert st == L.OK, st
        assert 0 < need.value <= L.STATIC_SCRATCH_BYTES
        stream.synchronize()
        cells = np.frombuffer(d_cells.cpu().numpy().tobytes(), dtype=CELL).reshape(len(prns), n_dop)
        np.testing.assert_array_equal(cells["index"], ref_cells["index"], err_msg=f"{name} call {call}")
        for f in ("level", "mean", "std"):
            np.testing.assert_allclose(cells[f], ref_cells[f], rtol=RTOL, err_msg=f"{name} call {call} {f}")


def test_static_entry_rejects_oversized_job(acq_golden):
    torch = pytest.importorskip("torch")
    lib = L.load()
    raw = acq_golden["acq_raw"]
    dev = torch.device("cuda", 0)
    d_raw = torch.from_numpy(raw.copy()).to(dev)
    d_codes = torch.zeros(N * 4, dtype=torch.float32, device=dev)
    d_cells = torch.zeros(4 * 4, dtype=torch.float32, device=dev)
    # 10 blocks x 401 Doppler bins x 4000 samples of spectra: about 128 MB > 16 MB
    job = L.StaticJob(d_raw.data_ptr(), L.SAMPLES_CI8, raw.shape[0], FS, 0.0, N, 10, 0, 1, 5000.0, 25.0,
                      d_codes.data_ptr(), 4, L.STAT_ABS, L.SPECTRUM_ONE_SIDED)
    need = C.c_size_t()
    st = lib.ugsdr_acquire_static(None, C.byref(job), C.c_void_p(d_cells.data_ptr()), C.byref(need))
    assert st == L.E_NOMEM
    assert need.value > L.STATIC_SCRATCH_BYTES
