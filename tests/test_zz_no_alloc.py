"""GPU: the allocation-free FFT entry point (SRX_fftLinesNoAlloc).

Callers that may not allocate device memory (code inside a CUDA graph
capture, real-time acquisition loops, plug-in hosts that own the device's
memory) use SRX_fftLinesNoAlloc, which stages its lines and twiddles in a
fixed file-scope device array instead of calling cudaMalloc.  This test calls
it through the C ABI, twice in a row, and checks each result against the
allocating entry point SRX_fftSelfTest (same kernel) within the FFT tests'
tolerance; it also checks that oversized requests are refused.

The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import cudasirecon_gb300 as sr

pytestmark = pytest.mark.gpu


def _lib():
    lib = sr.load_library()
    lib.SRX_fftLinesNoAlloc.restype = C.c_int
    lib.SRX_fftLinesNoAlloc.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int, C.c_int,
                                        C.c_int]
    lib.SRX_fftLinesNoAllocError.restype = C.c_char_p
    lib.SRX_fftLinesNoAllocError.argtypes = []
    return lib


def _noalloc(lib, x, inverse, columns):
    x = np.ascontiguousarray(x, np.complex64)
    out = np.empty_like(x)
    nl, n = x.shape
    rc = lib.SRX_fftLinesNoAlloc(x.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)),
                                 out.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)), n, nl, int(inverse),
                                 int(columns))
    assert rc == 0, lib.SRX_fftLinesNoAllocError()
    return out


@pytest.mark.parametrize("n,nl,inverse,columns", [(1024, 64, False, False), (48, 512, True, True),
                                                  (768, 8, True, False), (96, 4096, False, True),
                                                  (2048, 16, True, False)])
def test_no_alloc_matches_allocating_entry_point(n, nl, inverse, columns):
    lib = _lib()
    rng = np.random.default_rng(n + nl)
    x = (rng.standard_normal((nl, n)) + 1j * rng.standard_normal((nl, n))).astype(np.complex64)
    ref = sr.fft_selftest(x, inverse=inverse, columns=columns)
    tol = 2e-6 * max(1.0, np.log2(n))
    for _ in range(2):
        out = _noalloc(lib, x, inverse, columns)
        err = np.abs(out - ref).max() / np.abs(ref).max()
        assert err < tol, err


def test_no_alloc_rejects_oversized_requests():
    lib = _lib()
    x = np.zeros((1 << 12, 1024), np.complex64)  # 4 Mi values > 2 Mi limit
    out = np.empty_like(x)
    rc = lib.SRX_fftLinesNoAlloc(x.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)),
                                 out.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)), 1024, 1 << 12, 0, 0)
    assert rc != 0
    assert b"limit" in lib.SRX_fftLinesNoAllocError()
