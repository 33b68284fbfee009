"""The allocation-free entry point ugsdr_acquire_static.

Callers that cannot allocate device memory themselves (real-time receiver
loops that must not block on cudaMalloc, and host applications whose device
memory belongs to another allocator or pool) pass device pointers for inputs
and outputs; the library's scratch is a fixed-size file-scope device array.
This test calls it through the C ABI twice in a row and checks its cells
against ugsdr_acquire's on the same input (index exact, level/mean/std within
1e-4 relative), and that a job beyond the scratch limit is rejected.  It sits
in a file of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest

from conftest import unpack_codes
from ugsdr_gb300 import _lib as L

pytestmark = pytest.mark.gpu
RTOL = 1e-4


def static_job(d_raw, n_samples, d_codes, n_codes, n=4000, k=10, rng=5000.0, step=500.0):
    return L.StaticJob(d_raw.data_ptr(), L.SAMPLES_CI8, n_samples, 4e6, 0.0, n, k, 0, 1, rng, step,
                       d_codes.data_ptr(), n_codes, L.STAT_ABS, L.SPECTRUM_ONE_SIDED)


def test_static_entry_matches_acquire(ctx, acq_golden, golden_codes):
    torch = pytest.importorskip("torch")
    lib = L.load()
    ca = unpack_codes(golden_codes, "gps_l1ca")
    raw = acq_golden["acq_raw"]
    prns = [int(p) for p in acq_golden["acq_prns"]]
    from ugsdr_gb300 import api
    code_samples = np.stack([api.repeat_upsample(ca[p], 1, 4000) for p in prns]).astype(np.float32)

    # reference entry: ugsdr_acquire with its own context allocations
    hs = [ctx.code_put(ca[p], 4000) for p in prns]
    try:
        _, ref_cells = ctx.acquire(ctx.make_job(raw, L.SAMPLES_CI8, 4e6, 4000, 10, hs, 5000, 500), cells=True)
    finally:
        for h in hs:
            ctx.code_release(h)

    dev = torch.device("cuda", 0)
    d_raw = torch.from_numpy(raw.copy()).to(dev)
    d_codes = torch.from_numpy(code_samples).to(dev)
    n_dop = ref_cells.shape[1]
    d_cells = torch.zeros(len(prns) * n_dop * 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    job = static_job(d_raw, raw.shape[0], d_codes, len(prns))
    for call in range(2):
        d_cells.fill_(-1.0)
        need = C.c_size_t()
        torch.cuda.synchronize()
        st = lib.ugsdr_acquire_static(C.c_void_p(stream.cuda_stream), C.byref(job), C.c_void_p(d_cells.data_ptr()),
                                      C.byref(need))
        assert st == L.OK, st
        assert 0 < need.value <= L.STATIC_SCRATCH_BYTES
        stream.synchronize()
        cells = np.frombuffer(d_cells.cpu().numpy().tobytes(),
                              dtype=np.dtype([("level", "<f4"), ("index", "<u4"), ("mean", "<f4"), ("std", "<f4")]))
        cells = cells.reshape(len(prns), n_dop)
        np.testing.assert_array_equal(cells["index"], ref_cells["index"], err_msg=f"call {call}")
        for f in ("level", "mean", "std"):
            np.testing.assert_allclose(cells[f], ref_cells[f], rtol=RTOL, err_msg=f"call {call} {f}")


def test_static_entry_rejects_oversized_job(acq_golden):
    torch = pytest.importorskip("torch")
    lib = L.load()
    raw = acq_golden["acq_raw"]
    dev = torch.device("cuda", 0)
    d_raw = torch.from_numpy(raw.copy()).to(dev)
    d_codes = torch.zeros(4000 * 4, dtype=torch.float32, device=dev)
    d_cells = torch.zeros(4 * 4, dtype=torch.float32, device=dev)
    # 10 blocks x 401 Doppler bins x 4000 samples of spectra: about 128 MB > 16 MB
    job = static_job(d_raw, raw.shape[0], d_codes, 4, rng=5000.0, step=25.0)
    need = C.c_size_t()
    st = lib.ugsdr_acquire_static(None, C.byref(job), C.c_void_p(d_cells.data_ptr()), C.byref(need))
    assert st == L.E_NOMEM
    assert need.value > L.STATIC_SCRATCH_BYTES
