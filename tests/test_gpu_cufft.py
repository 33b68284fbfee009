"""cuFFT as the cross-check of the project's transforms (never on the
product path): ugsdr_dft — the single-CTA Stockham plans and, above one CTA,
the four-step kernels the acquisition path runs — against torch.fft on the
GPU (cuFFT) and numpy's FP64 FFT, at the block sizes of the configurations.
Bar: the project's error against FP64 (max |error| / max |X|) below 1e-5,
a tenth of the acquisition path's 1e-4; both errors and their ratio are
printed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [2046, 4000, 16000, 50000, 200000, 204600, 1_000_000]


@pytest.mark.parametrize("n", SIZES)
def test_dft_against_cufft(ctx, n):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    ours = ctx.dft(x)
    cufft = torch.fft.fft(torch.from_numpy(x).cuda()).cpu().numpy()
    ref = np.fft.fft(x.astype(np.complex128))
    scale = np.abs(ref).max()
    e_ours = np.abs(ours - ref).max() / scale
    e_cufft = np.abs(cufft - ref).max() / scale
    e_pair = np.abs(ours - cufft).max() / scale
    print(f"N={n}: project {e_ours:.2e}, cuFFT {e_cufft:.2e}, project vs cuFFT {e_pair:.2e} (of max |X|)")
    assert e_ours < 1e-5
