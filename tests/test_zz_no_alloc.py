"""GPU: the allocation-free FFT entry point (SRX_fftLinesNoAlloc).

Callers that may not allocate device memory (real-time acquisition loops,
where an allocation's implicit synchronisation stalls the camera pipeline,
and plug-in hosts that own the device's memory) use SRX_fftLinesNoAlloc,
which stages its lines and twiddles in a fixed file-scope device array
instead of calling cudaMalloc.  This test calls it through the C ABI, twice in
a row per case, and checks each result against the allocating entry point
SRX_fftSelfTest (same kernel) and against numpy's FP64 FFT, within the FFT
tests' tolerance.  It also checks that repeated calls leave the device's free
memory unchanged, and that refused requests leave the output untouched.

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
    lib.SRX_deviceMemInfo.restype = C.c_int
    lib.SRX_deviceMemInfo.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    return lib


def _call(lib, x, out, n, nl, inverse, columns):
    return lib.SRX_fftLinesNoAlloc(x.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)),
                                   out.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)), n, nl, int(inverse),
                                   int(columns))


def _noalloc(lib, x, inverse, columns):
    x = np.ascontiguousarray(x, np.complex64)
    out = np.empty_like(x)
    nl, n = x.shape
    rc = _call(lib, x, out, n, nl, inverse, columns)
    assert rc == 0, lib.SRX_fftLinesNoAllocError()
    return out


def _free_bytes(lib):
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert lib.SRX_deviceMemInfo(C.byref(free), C.byref(total)) == 0
    return free.value


# rows up to the 8192-point limit; columns up to 7168 points (the longest
# 2-3-5-7 length whose column staging fits one CTA's 227 KB of shared memory)
CASES = [(1024, 64, False, False), (48, 512, True, True), (768, 8, True, False), (96, 4096, False, True),
         (2048, 16, True, False), (4096, 8, False, False), (8192, 4, True, False), (8192, 2, False, False),
         (7168, 2, False, True), (4096, 4, True, True)]


@pytest.mark.parametrize("n,nl,inverse,columns", CASES)
def test_no_alloc_matches_allocating_entry_point_and_fp64(n, nl, inverse, columns):
    lib = _lib()
    rng = np.random.default_rng(n + nl)
    x = (rng.standard_normal((nl, n)) + 1j * rng.standard_normal((nl, n))).astype(np.complex64)
    ref = sr.fft_selftest(x, inverse=inverse, columns=columns)
    x64 = x.astype(np.complex128)
    exact = np.fft.ifft(x64, axis=1) * n if inverse else np.fft.fft(x64, axis=1)
    tol = 2e-6 * max(1.0, np.log2(n))
    for _ in range(2):
        out = _noalloc(lib, x, inverse, columns)
        err = np.abs(out - ref).max() / np.abs(ref).max()
        assert err < tol, f"vs SRX_fftSelfTest: {err:.3e}"
        err64 = np.abs(out - exact).max() / np.abs(exact).max()
        assert err64 < tol, f"vs numpy FP64: {err64:.3e}"


def test_no_alloc_leaves_device_memory_unchanged():
    lib = _lib()
    rng = np.random.default_rng(7)
    x = (rng.standard_normal((64, 1024)) + 1j * rng.standard_normal((64, 1024))).astype(np.complex64)
    _noalloc(lib, x, False, False)  # first call: address lookup, kernel attributes
    before = _free_bytes(lib)
    for inverse, columns in ((False, False), (True, False), (False, True), (True, True)):
        _noalloc(lib, x, inverse, columns)
    assert _free_bytes(lib) == before


@pytest.mark.parametrize("n,nl,columns,what", [(1024, 1 << 12, False, b"limit"), (16384, 1, False, b"limit"),
                                               (8192, 1, True, b"column"), (1000 + 1, 4, False, b"factor")])
def test_no_alloc_refuses_and_leaves_output_untouched(n, nl, columns, what):
    lib = _lib()
    x = np.ones((nl, n), np.complex64)
    out = np.full((nl, n), 123.5 - 7j, np.complex64)
    rc = _call(lib, x, out, n, nl, False, columns)
    assert rc != 0
    assert what in lib.SRX_fftLinesNoAllocError()
    assert np.all(out == np.complex64(123.5 - 7j))
