"""GPU: the shared-memory Stockham FFT engine against numpy for every radix
combination the reconstruction uses (2, 3, 4, 5, 7, 8, 16, 32 stages), both
directions and both shared-memory layouts."""
import numpy as np
import pytest

import cudasirecon_gb300 as sr

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 15, 16, 20, 24, 25, 32, 48, 49, 64, 80, 96, 128, 160, 192, 256,
         384, 512, 640, 768, 1024, 1536, 2048, 4096]


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("inverse", [False, True])
@pytest.mark.parametrize("columns", [False, True])
def test_fft_engine(n, inverse, columns):
    rng = np.random.default_rng(n)
    nl = max(1, min(8, 4096 // n)) * 2
    x = (rng.standard_normal((nl, n)) + 1j * rng.standard_normal((nl, n))).astype(np.complex64)
    y = sr.fft_selftest(x, inverse=inverse, columns=columns)
    ref = np.fft.ifft(x.astype(np.complex128), axis=1) * n if inverse else np.fft.fft(x.astype(np.complex128), axis=1)
    err = np.abs(y - ref).max() / max(np.abs(ref).max(), 1e-30)
    assert err < 2e-6 * max(1.0, np.log2(max(n, 2))), err
