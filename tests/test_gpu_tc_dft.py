"""ugsdr_dft25_batch: batched 25-point forward DFTs (the radix-25 butterfly of
the four-step inverse) on the CUDA cores and on the tensor cores (tcgen05,
3xTF32 split) against numpy's FP64 FFT.  Bars (max |error| over the batch /
max |y|): CUDA cores 1e-6, tensor cores 1e-5 — inside the acquisition path's
1e-4 relative bar with room for the other passes.  A batch that is not a
multiple of the 128-transform tile checks the partial tile."""
import ctypes as C

import numpy as np
import pytest

from ugsdr_gb300 import _lib as L

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method,bar", [(0, 1e-6), (1, 1e-5)])
def test_dft25_batch_vs_numpy(ctx, method, bar):
    torch = pytest.importorskip("torch")
    count = 100_003
    rng = np.random.default_rng(25)
    x = (rng.standard_normal((count, 25)) + 1j * rng.standard_normal((count, 25))).astype(np.complex64)
    d_in = torch.from_numpy(x.view(np.float32)).cuda()
    d_out = torch.full_like(d_in, float("nan"))
    ms = C.c_float()
    ctx._check(ctx.lib.ugsdr_dft25_batch(ctx.h, C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()), count, method,
                                         C.byref(ms)))
    y = d_out.cpu().numpy().view(np.complex64).reshape(count, 25)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    err = np.abs(y - ref).max() / np.abs(ref).max()
    print(f"method {method}: max error {err:.2e} of max |y|, {ms.value:.3f} ms for {count} transforms")
    assert np.isfinite(y).all() and err <= bar


def test_dft25_batch_rejects_bad_arguments(ctx):
    with pytest.raises(L.UgsdrError):
        ctx._check(ctx.lib.ugsdr_dft25_batch(ctx.h, None, None, 10, 0, None))
    with pytest.raises(L.UgsdrError):
        ctx._check(ctx.lib.ugsdr_dft25_batch(ctx.h, C.c_void_p(16), C.c_void_p(16), 10, 7, None))
