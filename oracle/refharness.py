"""ctypes driver for the reference harness library (test infrastructure only).

``oracle/_ref/librefsirecon.so`` is built by ``oracle/build_ref.py`` from the
reference's own GPU sources; this wrapper exposes the SR_* in-memory flow
(SR_new_from_shape -> SR_setRaw -> SR_loadAndRescaleImage -> SR_setCurTimeIdx
-> SR_processOneVolume -> SR_getResult, src/cudaSirecon/interface.cpp:13-45)
plus stage hooks used to capture intermediate bands.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_ref

_lib = None


def load(build: bool = True):
    global _lib
    if _lib is not None:
        return _lib
    path = build_ref.LIB
    if build or not os.path.exists(path):
        path = build_ref.build()
        if path is None:
            raise RuntimeError("reference harness could not be built")
    lib = C.CDLL(path)
    vp, fp, ip = C.c_void_p, C.POINTER(C.c_float), C.c_int
    lib.refh_new.restype = vp
    lib.refh_new.argtypes = [ip, ip, ip, C.c_char_p, fp, ip, ip, ip]
    lib.refh_delete.argtypes = [vp]
    for name in ("refh_set_ntimes", "refh_set_cur_time", "refh_load_and_rescale"):
        getattr(lib, name).argtypes = [vp, ip]
    lib.refh_set_raw.argtypes = [vp, fp]
    for name in ("refh_stage_separate", "refh_stage_fit", "refh_stage_assemble"):
        getattr(lib, name).argtypes = [vp]
    lib.refh_process.argtypes = [vp]
    lib.refh_process.restype = ip
    lib.refh_get_result.argtypes = [vp, fp]
    lib.refh_get_band.argtypes = [vp, ip, ip, fp]
    lib.refh_get_fit.argtypes = [vp, fp, fp]
    lib.refh_get_k0guess.argtypes = [vp, fp]
    lib.refh_norders.argtypes = [vp]
    lib.refh_norders.restype = ip
    lib.refh_nz.argtypes = [vp]
    lib.refh_nz.restype = ip
    lib.refh_nx.argtypes = [vp]
    lib.refh_nx.restype = ip
    lib.refh_set_section_backgrounds.argtypes = [vp, fp, ip]
    lib.refh_fit_counts.argtypes = [vp, C.POINTER(C.c_longlong)]
    lib.refh_capture_overlaps.argtypes = [vp, ip]
    lib.refh_get_captured.argtypes = [vp, ip, fp]
    lib.refh_get_captured.restype = C.c_longlong
    _lib = lib
    return lib


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class RefRecon:
    """One reference SIM_Reconstructor (in-memory construction path)."""

    def __init__(self, nx: int, ny: int, nimages: int, config: str, otf_pages: np.ndarray, ndirs: int = 3,
                 zoom: float = 2.0, z_zoom: int = 1):
        self.lib = load()
        self.otf = np.ascontiguousarray(otf_pages, np.float32)
        d, h, w = self.otf.shape
        self.h = self.lib.refh_new(nx, ny, nimages, config.encode(), _fptr(self.otf), w, h, d)
        self.nx_raw, self.ny, self.nimages, self.ndirs = nx, ny, nimages, ndirs
        self.nx = self.lib.refh_nx(self.h)  # after deskew / cropXY
        self.nz = self.lib.refh_nz(self.h)
        self.norders = self.lib.refh_norders(self.h)
        self.out_shape = (z_zoom * self.nz, int(round(zoom * ny)), int(round(zoom * self.nx)))

    def close(self):
        if self.h:
            self.lib.refh_delete(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_ntimes(self, n: int):
        self.lib.refh_set_ntimes(self.h, n)

    def set_raw(self, raw: np.ndarray):
        r = np.ascontiguousarray(raw, np.float32)
        assert r.shape == (self.nimages, self.ny, self.nx_raw), r.shape
        self.lib.refh_set_raw(self.h, _fptr(r))

    def set_section_backgrounds(self, values):
        """Per raw section extra background (the reference's bBgInExtHdr
        values from the MRC extended header)."""
        v = np.ascontiguousarray(values, np.float32)
        self.lib.refh_set_section_backgrounds(self.h, _fptr(v), v.size)

    def load_and_rescale(self, it: int = 0):
        self.lib.refh_load_and_rescale(self.h, it)

    def set_cur_time(self, it: int):
        self.lib.refh_set_cur_time(self.h, it)

    def stage_separate(self):
        self.lib.refh_stage_separate(self.h)

    def stage_fit(self):
        self.lib.refh_stage_fit(self.h)

    def stage_assemble(self):
        self.lib.refh_stage_assemble(self.h)

    def process(self):
        return self.lib.refh_process(self.h)

    def result(self) -> np.ndarray:
        out = np.empty(self.out_shape, np.float32)
        self.lib.refh_get_result(self.h, _fptr(out))
        return out

    def band(self, d: int, b: int) -> np.ndarray:
        nxh = self.nx // 2 + 1
        out = np.empty((self.nz, self.ny, nxh * 2), np.float32)
        self.lib.refh_get_band(self.h, d, b, _fptr(out))
        return out[..., 0::2] + 1j * out[..., 1::2]

    def fit(self):
        k0 = np.empty((self.ndirs, 2), np.float32)
        amp = np.empty((self.ndirs, self.norders, 2), np.float32)
        self.lib.refh_get_fit(self.h, _fptr(k0), _fptr(amp))
        return k0, amp[..., 0] + 1j * amp[..., 1]

    def capture_overlaps(self, on: bool = True):
        """Keep each direction's overlap pair right after findk0."""
        self.lib.refh_capture_overlaps(self.h, int(on))

    def captured_overlaps(self, d: int):
        """(overlap0, overlap1) of direction d after findk0, complex
        [nz][ny][nx] each, or None."""
        n = self.lib.refh_get_captured(self.h, d, None)
        if n == 0:
            return None
        buf = np.empty(n, np.float32)
        self.lib.refh_get_captured(self.h, d, _fptr(buf))
        c = buf[0::2] + 1j * buf[1::2]
        half = c.size // 2
        return c[:half].reshape(self.nz, self.ny, self.nx), c[half:].reshape(self.nz, self.ny, self.nx)

    def fit_counts(self) -> dict:
        """Overlap builds, reductions and k0 searches executed since creation."""
        c = (C.c_longlong * 3)()
        self.lib.refh_fit_counts(self.h, c)
        return {"overlap_builds": c[0], "reductions": c[1], "k0_searches": c[2]}

    def k0guess(self):
        k0 = np.empty((self.ndirs, 2), np.float32)
        self.lib.refh_get_k0guess(self.h, _fptr(k0))
        return k0
