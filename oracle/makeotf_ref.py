"""Runs the reference makeotf program (src/otf/radialft.cpp, compiled
unmodified by oracle/build_ref.py:build_makeotf into
oracle/_ref/libmakeotf_ref.so) on a PSF stack held in memory.

Test infrastructure only: the tests and the golden-fixture generator use it
to pin the makeotf oracle (oracle/makeotf_oracle.py).  The PSF goes in, and
the OTF comes back, through CImg's raw ".cimg" format, which the reference's
own CImg reads and writes without libtiff; FFTW's r2c transform is replaced
by a double-precision DFT (oracle/ref_harness/makeotf_harness.cpp).
"""
from __future__ import annotations

import ctypes
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libmakeotf_ref.so")
_lib = None


def write_cimg(path: str, vol: np.ndarray) -> None:
    """float32 [d][h][w] -> CImg raw file (one image, little endian)."""
    vol = np.ascontiguousarray(vol, dtype="<f4")
    if vol.ndim == 2:
        vol = vol[None]
    d, h, w = vol.shape
    with open(path, "wb") as f:
        f.write(b"1 float little_endian\n")
        f.write(f"{w} {h} {d} 1\n".encode())
        f.write(vol.tobytes())


def read_cimg(path: str) -> np.ndarray:
    """CImg raw file (one float image) -> float32 [d][h][w]."""
    with open(path, "rb") as f:
        head = f.readline().split()
        if int(head[0]) != 1 or head[1] != b"float" or head[2] != b"little_endian":
            raise ValueError(f"unexpected CImg header {head!r}")
        w, h, d, c = (int(v) for v in f.readline().split()[:4])
        data = np.frombuffer(f.read(w * h * d * c * 4), dtype="<f4")
    return data.reshape(c, d, h, w)[0].copy()


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            import build_ref  # type: ignore  # noqa: F401  (oracle/ on sys.path)
        _lib = ctypes.CDLL(LIB)
        _lib.mo_ref_main.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        _lib.mo_ref_main.restype = ctypes.c_int
    return _lib


def run(psf: np.ndarray, args: list[str]) -> np.ndarray:
    """makeotf <psf> <otf.tif> args...; returns the OTF file's float32 array
    [depth][height][width] = [norders][nx/2+1][2*nz] (complex kz along a
    row), exactly what the reference writes."""
    lib = load()
    with tempfile.TemporaryDirectory() as td:
        ipath = os.path.join(td, "psf.cimg")
        opath = os.path.join(td, "otf.tif")
        write_cimg(ipath, psf)
        argv = [b"makeotf", ipath.encode(), opath.encode()] + [a.encode() for a in args]
        arr = (ctypes.c_char_p * len(argv))(*argv)
        rc = lib.mo_ref_main(len(argv), arr)
        if rc != 0:
            raise RuntimeError(f"reference makeotf exited with {rc}")
        return read_cimg(opath)
