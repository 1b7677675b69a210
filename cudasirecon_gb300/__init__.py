"""cudasirecon_gb300: GB300-native 3-beam SIM reconstruction.

The product is ``libcudasirecon.so`` (C++ host code + hand-written sm_103a
CUDA kernels) exposing the reference's SR_* C ABI (include/cudasirecon.h).
This module is a thin ctypes mirror of that ABI for Python callers, tests
and benchmarks.  There is no CPU fallback: if the library is missing or the
GPU is unavailable, calls fail loudly.
"""
from __future__ import annotations

import ctypes as C
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcudasirecon.so")
CLI_PATH = os.path.join(HERE, "bin", "cudasirecon")

_lib = None


class SIReconError(RuntimeError):
    pass


def build(force: bool = False) -> str:
    from . import buildlib
    return buildlib.build(force=force)


class BatchItem(C.Structure):
    """SRX_BatchItem (include/cudasirecon.h)."""
    _fields_ = [("config", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nimages", C.c_int),
                ("raw", C.c_void_p), ("raw_is_u16", C.c_int), ("out", C.c_void_p)]


def load_library(path: str | None = None) -> C.CDLL:
    """Load libcudasirecon.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise SIReconError(f"{path} not found: build it with `python -m cudasirecon_gb300.buildlib`")
    lib = C.CDLL(path)
    vp, ip, fp = C.c_void_p, C.c_int, C.POINTER(C.c_float)
    lib.SR_new_from_shape.restype = vp
    lib.SR_new_from_shape.argtypes = [ip, ip, ip, C.c_char_p]
    lib.SR_new_from_argv.restype = vp
    lib.SR_new_from_argv.argtypes = [ip, C.POINTER(C.c_char_p)]
    lib.SR_setRaw.argtypes = [vp, fp, ip, ip, ip]
    lib.SR_setRawU16.argtypes = [vp, C.POINTER(C.c_uint16), ip, ip, ip]
    for n in ("SR_loadAndRescaleImage", "SR_setFile", "SR_writeResult"):
        getattr(lib, n).argtypes = [vp, ip, ip]
    lib.SR_setCurTimeIdx.argtypes = [vp, ip]
    for n in ("SR_processOneVolume", "SR_closeFiles", "SR_delete"):
        getattr(lib, n).argtypes = [vp]
    lib.SR_getResult.argtypes = [vp, fp]
    lib.SR_getReconParams.restype = vp
    lib.SR_getReconParams.argtypes = [vp]
    lib.SR_getImageParams.restype = vp
    lib.SR_getImageParams.argtypes = [vp]
    lib.SR_getLastError.restype = C.c_char_p
    lib.SR_getLastError.argtypes = []
    lib.SR_clearError.argtypes = []
    lib.SR_getNTimes.restype = ip
    lib.SR_getNTimes.argtypes = [vp]
    lib.SRX_getFit.argtypes = [vp, fp, fp]
    lib.SRX_prepare.restype = ip
    lib.SRX_prepare.argtypes = [vp]
    lib.SRX_getBand.restype = ip
    lib.SRX_getBand.argtypes = [vp, ip, ip, fp]
    lib.SRX_benchDevice.restype = ip
    lib.SRX_benchDevice.argtypes = [vp, ip, C.POINTER(C.c_double)]
    lib.SRX_setProfiling.argtypes = [vp, ip]
    lib.SRX_fitCounts.restype = None
    lib.SRX_fitCounts.argtypes = [vp, C.POINTER(C.c_longlong)]
    lib.SRX_tuneFFT.restype = ip
    lib.SRX_tuneFFT.argtypes = [vp, ip, C.c_char_p, ip]
    lib.SRX_fftPlanChoice.restype = ip
    lib.SRX_fftPlanChoice.argtypes = [ip, ip, C.c_char_p, ip]
    lib.SRX_setFilterFusion.restype = None
    lib.SRX_setFilterFusion.argtypes = [vp, ip]
    lib.SRX_setDeviceK0Search.restype = None
    lib.SRX_setDeviceK0Search.argtypes = [vp, ip]
    lib.SRX_getProfile.restype = ip
    lib.SRX_getProfile.argtypes = [vp, C.c_char_p, ip]
    lib.SRX_resetProfile.argtypes = [vp]
    lib.SRX_kernelLaunches.restype = C.c_longlong
    lib.SRX_kernelLaunches.argtypes = [vp]
    lib.SRX_fftSelfTest.restype = ip
    lib.SRX_fftSelfTest.argtypes = [fp, ip, ip, ip, ip]
    lib.SRX_pinHost.restype = ip
    lib.SRX_pinHost.argtypes = [vp, C.c_size_t]
    lib.SRX_unpinHost.restype = ip
    lib.SRX_unpinHost.argtypes = [vp]
    lib.SRX_hostAlloc.restype = vp
    lib.SRX_hostAlloc.argtypes = [C.c_size_t]
    lib.SRX_hostFree.restype = None
    lib.SRX_hostFree.argtypes = [vp]
    lib.SRX_processSeries.restype = ip
    lib.SRX_processSeries.argtypes = [vp, C.POINTER(vp), ip, C.POINTER(vp), ip, ip]
    lib.SRX_serverCreate.restype = vp
    lib.SRX_serverCreate.argtypes = [ip, C.c_size_t]
    lib.SRX_serverAddConfig.restype = ip
    lib.SRX_serverAddConfig.argtypes = [vp, C.c_char_p]
    lib.SRX_serverSubmit.restype = C.c_longlong
    lib.SRX_serverSubmit.argtypes = [vp, ip, ip, ip, ip, vp, ip, vp]
    lib.SRX_serverWait.restype = ip
    lib.SRX_serverWait.argtypes = [vp, C.c_longlong, C.POINTER(C.c_double)]
    lib.SRX_serverReserve.restype = ip
    lib.SRX_serverReserve.argtypes = [vp, ip, ip, ip, ip, ip]
    lib.SRX_serverRunBatch.restype = ip
    lib.SRX_batchPlan.restype = ip
    lib.SRX_batchPlan.argtypes = [C.POINTER(BatchItem), ip, ip, C.POINTER(C.c_int)]
    lib.SRX_serverRunBatch.argtypes = [vp, C.POINTER(BatchItem), ip]
    lib.SRX_serverDeviceBytes.restype = C.c_size_t
    lib.SRX_serverSetK0Reuse.restype = ip
    lib.SRX_serverSetK0Reuse.argtypes = [vp, ip, ip]
    lib.SRX_serverRecordedK0.restype = ip
    lib.SRX_serverRecordedK0.argtypes = [vp, ip, C.POINTER(C.c_float), ip]
    lib.SRX_serverCounters.restype = None
    lib.SRX_serverCounters.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    lib.SRX_serverDeviceBytes.argtypes = [vp]
    lib.SRX_serverDeviceBytesHeld.restype = C.c_size_t
    lib.SRX_serverDeviceBytesHeld.argtypes = [vp]
    lib.SRX_serverMemory.restype = None
    lib.SRX_serverMemory.argtypes = [vp, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    lib.SRX_serverPlannedBytes.restype = C.c_size_t
    lib.SRX_serverPlannedBytes.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
    lib.SRX_serverAdmissionWaits.restype = C.c_longlong
    lib.SRX_serverAdmissionWaits.argtypes = [vp]
    lib.SRX_serverDestroy.argtypes = [vp]
    lib.SRX_makeOTF.restype = ip
    lib.SRX_makeOTF.argtypes = [fp, ip, ip, ip, ip, C.POINTER(C.c_char_p), fp, C.c_size_t, C.POINTER(C.c_int)]
    lib.SRX_makeotfMain.restype = ip
    lib.SRX_makeotfMain.argtypes = [ip, C.POINTER(C.c_char_p)]
    _lib = lib
    return lib


class ImageParams(C.Structure):
    """ctypes view of ImageParams (cudaSireconImpl.h:179-195 layout)."""
    _fields_ = [("nx", C.c_int), ("nx_raw", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("nz0", C.c_int),
                ("nwaves", C.c_short), ("wave", C.c_short * 5), ("ntimes", C.c_short),
                ("curTimeIdx", C.c_ushort), ("dxy", C.c_float), ("dz", C.c_float), ("dz_raw", C.c_float),
                ("inscale", C.c_float)]


class ReconParamsHead(C.Structure):
    """ctypes view of the leading plain members of ReconParams (up to wienerInr)."""
    _fields_ = [("k0startangle", C.c_float), ("linespacing", C.c_float), ("na", C.c_float), ("nimm", C.c_float),
                ("ndirs", C.c_int), ("nphases", C.c_int), ("norders_output", C.c_int), ("norders", C.c_int),
                ("phaseSteps", C.c_void_p), ("bTwolens", C.c_bool), ("bFastSIM", C.c_bool), ("bBessel", C.c_bool),
                ("BesselNA", C.c_float), ("BesselLambdaEx", C.c_float), ("deskewAngle", C.c_float),
                ("extraShift", C.c_int), ("bNoRecon", C.c_bool), ("cropXYto", C.c_uint), ("bWriteTitle", C.c_bool),
                ("otfcutoff", C.c_float), ("zoomfact", C.c_float), ("z_zoom", C.c_int), ("nzPadTo", C.c_int),
                ("explodefact", C.c_float), ("bFilteroverlaps", C.c_bool), ("recalcarrays", C.c_int),
                ("napodize", C.c_int), ("bSearchforvector", C.c_int), ("bUseTime0k0", C.c_int),
                ("apodizeoutput", C.c_int), ("apoGamma", C.c_float), ("bSuppress_singularities", C.c_int),
                ("suppression_radius", C.c_int), ("bDampenOrder0", C.c_bool), ("bFitallphases", C.c_int),
                ("do_rescale", C.c_int), ("equalizez", C.c_bool), ("equalizet", C.c_bool), ("bNoKz0", C.c_bool),
                ("wiener", C.c_float), ("wienerInr", C.c_float)]


def write_tiff_float(path: str, pages: np.ndarray) -> None:
    """Write a float32 stack [depth][height][width] as an uncompressed multi-page TIFF."""
    pages = np.ascontiguousarray(pages, np.float32)
    if pages.ndim == 2:
        pages = pages[None]
    d, h, w = pages.shape
    import struct
    out = bytearray(b"II*\x00" + struct.pack("<I", 8))
    for p in range(d):
        ntags = 10
        data_off = len(out) + 2 + 12 * ntags + 4
        nbytes = w * h * 4
        nxt = data_off + nbytes if p + 1 < d else 0
        ent = b"".join([
            struct.pack("<HHII", 256, 4, 1, w), struct.pack("<HHII", 257, 4, 1, h),
            struct.pack("<HHIHH", 258, 3, 1, 32, 0), struct.pack("<HHIHH", 259, 3, 1, 1, 0),
            struct.pack("<HHIHH", 262, 3, 1, 1, 0), struct.pack("<HHII", 273, 4, 1, data_off),
            struct.pack("<HHIHH", 277, 3, 1, 1, 0), struct.pack("<HHII", 278, 4, 1, h),
            struct.pack("<HHII", 279, 4, 1, nbytes), struct.pack("<HHIHH", 339, 3, 1, 3, 0)])
        out += struct.pack("<H", ntags) + ent + struct.pack("<I", nxt)
        out += pages[p].tobytes()
    with open(path, "wb") as f:
        f.write(out)


def read_tiff_float(path: str) -> np.ndarray:
    """Read an uncompressed little-endian 32-bit float multi-page TIFF (any
    strip layout) into float32 [depth][height][width]."""
    import struct
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:4] != b"II*\x00":
        raise ValueError("not a little-endian classic TIFF")
    (off,) = struct.unpack_from("<I", buf, 4)
    pages = []
    while off:
        (n,) = struct.unpack_from("<H", buf, off)
        tags = {}
        for i in range(n):
            tag, typ, cnt, val = struct.unpack_from("<HHII", buf, off + 2 + 12 * i)
            size = {3: 2, 4: 4}.get(typ, 4)
            if cnt * size <= 4:
                fmt = "<" + ("H" if typ == 3 else "I") * cnt
                vals = list(struct.unpack_from(fmt, buf, off + 2 + 12 * i + 8))
            else:
                vals = list(struct.unpack_from("<" + ("H" if typ == 3 else "I") * cnt, buf, val))
            tags[tag] = vals
        w, h = tags[256][0], tags[257][0]
        if tags.get(258, [32])[0] != 32 or tags.get(259, [1])[0] != 1 or tags.get(339, [3])[0] != 3:
            raise ValueError("only uncompressed float32 TIFF pages are supported")
        data = b"".join(buf[o:o + c] for o, c in zip(tags[273], tags[279]))
        pages.append(np.frombuffer(data, "<f4", count=w * h).reshape(h, w))
        (off,) = struct.unpack_from("<I", buf, off + 2 + 12 * n)
    return np.stack(pages).astype(np.float32)


def _err(lib) -> str:
    return (lib.SR_getLastError() or b"").decode(errors="replace")


class Reconstructor:
    """One SIM_Reconstructor through the C ABI (SR_new_from_shape path).

    ``config`` is the reference's key=value config text (or a path); the OTF
    is given as TIFF pages (written to a temporary file and named with
    ``otf-file=``) or as an existing ``otf_path``.
    """

    def __init__(self, nx: int, ny: int, nimages: int, config: str, otf_pages: np.ndarray | None = None,
                 otf_path: str | None = None):
        self.lib = load_library()
        self._tmp = tempfile.TemporaryDirectory(prefix="sirecon_")
        if otf_path is None:
            otf_path = os.path.join(self._tmp.name, "otf.tif")
            write_tiff_float(otf_path, otf_pages)
        text = config if "=" in config else open(config).read()
        cfg = os.path.join(self._tmp.name, "config.txt")
        with open(cfg, "w") as f:
            f.write(text.rstrip("\n") + f"\notf-file={otf_path}\n")
        self.lib.SR_clearError()
        self.h = self.lib.SR_new_from_shape(nx, ny, nimages, cfg.encode())
        if not self.h:
            raise SIReconError(_err(self.lib))
        self.nx, self.ny, self.nimages = nx, ny, nimages  # the raw planes' shape
        ip = self.image_params()
        rp = self.recon_params()
        self.nz = ip.nz
        self.ndirs = rp.ndirs
        self.nphases = rp.nphases
        self.norders = rp.norders
        self.nx_recon = ip.nx  # after deskew / cropXY
        self.out_shape = (rp.z_zoom * ip.nz0, int(round(rp.zoomfact * ny)), int(round(rp.zoomfact * ip.nx)))

    def _check(self):
        e = _err(self.lib)
        if e:
            self.lib.SR_clearError()
            raise SIReconError(e)

    def close(self):
        if getattr(self, "h", None):
            self.lib.SR_delete(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def image_params(self) -> ImageParams:
        return ImageParams.from_address(self.lib.SR_getImageParams(self.h))

    def recon_params(self) -> ReconParamsHead:
        return ReconParamsHead.from_address(self.lib.SR_getReconParams(self.h))

    def set_raw(self, raw: np.ndarray):
        raw = np.ascontiguousarray(raw)
        if raw.dtype == np.uint16:
            self.lib.SR_setRawU16(self.h, raw.ctypes.data_as(C.POINTER(C.c_uint16)), self.nx, self.ny,
                                  raw.shape[0])
        else:
            raw = np.ascontiguousarray(raw, np.float32)
            self.lib.SR_setRaw(self.h, raw.ctypes.data_as(C.POINTER(C.c_float)), self.nx, self.ny, raw.shape[0])
        self._check()

    def load_and_rescale(self, it: int = 0, iw: int = 0):
        self.lib.SR_loadAndRescaleImage(self.h, it, iw)
        self._check()

    def set_cur_time(self, it: int):
        self.lib.SR_setCurTimeIdx(self.h, it)
        self._check()

    def process(self):
        self.lib.SR_processOneVolume(self.h)
        self._check()

    def result(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.out_shape, np.float32)
        self.lib.SR_getResult(self.h, out.ctypes.data_as(C.POINTER(C.c_float)))
        self._check()
        return out

    def fit(self):
        k0 = np.zeros((self.ndirs, 2), np.float32)
        amp = np.zeros((self.ndirs, self.norders, 2), np.float32)
        self.lib.SRX_getFit(self.h, k0.ctypes.data_as(C.POINTER(C.c_float)),
                            amp.ctypes.data_as(C.POINTER(C.c_float)))
        return k0, amp[..., 0] + 1j * amp[..., 1]

    def prepare(self):
        self.lib.SRX_prepare(self.h)
        self._check()

    def band(self, d: int, b: int) -> np.ndarray:
        nxh = self.nx_recon // 2 + 1
        out = np.empty((self.nz, self.ny, nxh * 2), np.float32)
        self.lib.SRX_getBand(self.h, d, b, out.ctypes.data_as(C.POINTER(C.c_float)))
        self._check()
        return out[..., 0::2] + 1j * out[..., 1::2]

    def set_ntimes(self, n: int):
        self.image_params().ntimes = n

    def bench_device(self, steps: int) -> float:
        t = C.c_double(0)
        rc = self.lib.SRX_benchDevice(self.h, steps, C.byref(t))
        if rc != 0:
            self._check()
        return t.value

    def set_profiling(self, on: bool = True):
        self.lib.SRX_setProfiling(self.h, int(on))

    def fit_counts(self) -> dict:
        """Overlap builds, overlap-pair reductions and k0 searches executed
        since creation (SRX_fitCounts)."""
        c = (C.c_longlong * 3)()
        self.lib.SRX_fitCounts(self.h, c)
        return {"overlap_builds": c[0], "reductions": c[1], "k0_searches": c[2]}

    def tune_fft(self, reps: int = 2) -> dict:
        """Time both FFT paths at every site/length of this handle's volume on
        the staged raw stack and record the faster ones in the plan cache
        (SRX_tuneFFT)."""
        import json
        buf = C.create_string_buffer(1 << 16)
        n = self.lib.SRX_tuneFFT(self.h, int(reps), buf, len(buf))
        if n < 0:
            raise SIReconError(_err(self.lib))
        return json.loads(buf.value.decode())

    def set_filter_fusion(self, on: bool = True):
        """Wiener filter inside the assembly's band load (default) or as its
        own pass (SRX_setFilterFusion)."""
        self.lib.SRX_setFilterFusion(self.h, int(on))

    def set_device_search(self, on: bool = True):
        """k0 search on the device (default) or host-driven
        (SRX_setDeviceK0Search)."""
        self.lib.SRX_setDeviceK0Search(self.h, int(on))

    def profile(self) -> dict:
        import json
        buf = C.create_string_buffer(1 << 16)
        self.lib.SRX_getProfile(self.h, buf, len(buf))
        return json.loads(buf.value.decode() or "{}")

    def reset_profile(self):
        self.lib.SRX_resetProfile(self.h)

    def kernel_launches(self) -> int:
        return int(self.lib.SRX_kernelLaunches(self.h))

    def process_series(self, raws, outs, t0: int = 0) -> None:
        """SRX_processSeries: raws[i] (uint16 or float32 stacks of the setRaw
        shape) -> outs[i] (float32 result arrays), volume i at time t0+i, with
        uploads and downloads overlapped with the computation."""
        n = len(raws)
        if len(outs) != n:
            raise ValueError("raws and outs differ in length")
        u16 = raws[0].dtype == np.uint16
        for r in raws:
            if r.dtype != raws[0].dtype or not r.flags.c_contiguous or r.size != raws[0].size:
                raise ValueError("raw stacks must share dtype and size and be C-contiguous")
        for o in outs:
            if o.dtype != np.float32 or not o.flags.c_contiguous or o.size != self.out_shape[0] * self.out_shape[1] * \
                    self.out_shape[2]:
                raise ValueError("outputs must be C-contiguous float32 arrays of the result shape")
        rp = (C.c_void_p * n)(*[r.ctypes.data for r in raws])
        op = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
        if self.lib.SRX_processSeries(self.h, rp, int(u16), op, n, t0) != 0:
            raise SIReconError(_err(self.lib))


def pin(array: np.ndarray) -> None:
    """Page-lock a numpy array's memory (SRX_pinHost)."""
    lib = load_library()
    if lib.SRX_pinHost(array.ctypes.data, array.nbytes) != 0:
        raise SIReconError(_err(lib))


def unpin(array: np.ndarray) -> None:
    lib = load_library()
    lib.SRX_unpinHost(array.ctypes.data)


class _HostBlock:
    """Owner of one SRX_hostAlloc block; freed when the last view goes."""

    def __init__(self, lib, nbytes: int):
        self.lib = lib
        self.ptr = lib.SRX_hostAlloc(nbytes)
        if not self.ptr:
            raise SIReconError(_err(lib))

    def __del__(self):
        try:
            self.lib.SRX_hostFree(C.c_void_p(self.ptr))
        except Exception:
            pass


def host_empty(shape, dtype=np.float32) -> np.ndarray:
    """A numpy array in page-locked memory from the CUDA runtime
    (SRX_hostAlloc): the fastest source and destination for raw stacks and
    results.  The memory is freed with the array."""
    lib = load_library()
    dt = np.dtype(dtype)
    count = int(np.prod(shape))
    blk = _HostBlock(lib, count * dt.itemsize)
    buf = (C.c_char * max(count * dt.itemsize, 1)).from_address(blk.ptr)
    buf._owner = blk  # the block lives as long as the buffer, the buffer as long as the array
    return np.frombuffer(buf, dtype=dt, count=count).reshape(shape)


FFT_SITES = {"ingest_x": 0, "ingest_y": 1, "separate_z": 2, "overlap_x": 3, "overlap_y": 4, "crosscorr_rows": 5,
             "crosscorr_cols": 6, "assemble_y": 7, "assemble_x": 8, "assemble_z": 9, "makeotf": 10}


def fft_plan_choice(site: str, n: int):
    """(register path?, source) the FFT call site uses for length n."""
    lib = load_library()
    buf = C.create_string_buffer(64)
    r = lib.SRX_fftPlanChoice(FFT_SITES[site], int(n), buf, len(buf))
    if r < 0:
        raise SIReconError("unknown FFT site")
    return bool(r), buf.value.decode()


def fft_selftest(x: np.ndarray, inverse: bool = False, columns: bool = False) -> np.ndarray:
    """Run the library's FFT engine on lines x[nlines][n] (complex64)."""
    lib = load_library()
    a = np.ascontiguousarray(x, np.complex64).copy()
    nl, n = a.shape
    rc = lib.SRX_fftSelfTest(a.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)), n, nl, int(inverse),
                             int(columns))
    if rc != 0:
        raise SIReconError(_err(lib) or f"fft self test failed ({rc})")
    return a


def make_otf(psf: np.ndarray, args: list[str] | tuple = ()) -> np.ndarray:
    """makeotf on the GPU (SRX_makeOTF): PSF stack float [nz*nphases][ny][nx]
    (phase fastest) and makeotf switches -> the OTF file's float array
    [bands][nx/2+1][2*nz] ([bands][1][2*(nx/2+1)] for a 2D PSF)."""
    lib = load_library()
    p = np.ascontiguousarray(psf, np.float32)
    nsec, ny, nx = p.shape
    args = list(args)
    argv = (C.c_char_p * max(1, len(args)))(*[a.encode() for a in args])
    nph = int(args[args.index("-nphases") + 1]) if "-nphases" in args else 5
    nz = max(1, nsec // max(1, nph))
    nb = nph if "-5bands" in args else (nph + 1) // 2
    shape = (nb, nx // 2 + 1, 2 * nz) if nz > 1 else (nb, 1, 2 * (nx // 2 + 1))
    out = np.empty(shape, np.float32)
    dims = (C.c_int * 3)()
    f32p = C.POINTER(C.c_float)
    if lib.SRX_makeOTF(p.ctypes.data_as(f32p), nx, ny, nsec, len(args), argv, out.ctypes.data_as(f32p), out.size,
                       dims) != 0:
        raise SIReconError(_err(lib))
    if (dims[2], dims[1], dims[0]) != out.shape:
        raise SIReconError(f"unexpected OTF shape {tuple(dims)}")
    return out


def makeotf_main(argv: list[str]) -> None:
    """The makeotf program (SRX_makeotfMain) in-process: argv without the
    program name, e.g. ["psf.tif", "otf.tif", "-angle", "-0.8", ...]."""
    lib = load_library()
    full = ["makeotf"] + list(argv)
    arr = (C.c_char_p * len(full))(*[a.encode() for a in full])
    if lib.SRX_makeotfMain(len(full), arr) != 0:
        raise SIReconError(_err(lib))


class Server:
    """SRX_server*: volumes of several shapes and acquisition configurations
    served concurrently by worker threads over pooled handles, within a
    device-memory budget.  Each request is processed as a time-0 volume."""

    def __init__(self, workers: int = 6, hbm_budget: float = 150e9):
        self.lib = load_library()
        self._tmp = tempfile.TemporaryDirectory(prefix="sirecon_srv_")
        self.lib.SR_clearError()
        self.h = self.lib.SRX_serverCreate(int(workers), int(hbm_budget))
        if not self.h:
            raise SIReconError(_err(self.lib))
        self._keep = {}
        self._n = 0

    def add_config(self, config: str, otf_pages: np.ndarray) -> int:
        """config: reference key=value text; otf_pages: the OTF TIFF's pages."""
        self._n += 1
        otf = os.path.join(self._tmp.name, f"otf{self._n}.tif")
        write_tiff_float(otf, otf_pages)
        cfg = os.path.join(self._tmp.name, f"config{self._n}.txt")
        with open(cfg, "w") as f:
            f.write(config.rstrip("\n") + f"\notf-file={otf}\n")
        cid = self.lib.SRX_serverAddConfig(self.h, cfg.encode())
        if cid < 0:
            raise SIReconError(_err(self.lib))
        return cid

    def submit(self, config: int, raw: np.ndarray, out: np.ndarray) -> int:
        """raw: [nimages][ny][nx] uint16 or float32 (C-contiguous); out: float32
        array of the result size.  Both must stay alive until wait()."""
        if not raw.flags.c_contiguous or not out.flags.c_contiguous or out.dtype != np.float32:
            raise ValueError("raw and out must be C-contiguous, out float32")
        if raw.dtype not in (np.uint16, np.float32) or raw.ndim != 3:
            raise ValueError("raw must be a [nimages][ny][nx] uint16 or float32 array")
        nimg, ny, nx = raw.shape
        t = self.lib.SRX_serverSubmit(self.h, config, nx, ny, nimg, raw.ctypes.data, int(raw.dtype == np.uint16),
                                      out.ctypes.data)
        if t < 0:
            raise SIReconError(_err(self.lib))
        self._keep[t] = (raw, out)
        return int(t)

    def wait(self, ticket: int) -> float:
        """Blocks until the request is done; returns its latency in ms."""
        lat = C.c_double(0.0)
        rc = self.lib.SRX_serverWait(self.h, ticket, C.byref(lat))
        self._keep.pop(ticket, None)
        if rc != 0:
            raise SIReconError(_err(self.lib))
        return lat.value

    def reserve(self, config: int, nx: int, ny: int, nimages: int, count: int) -> int:
        """Create `count` handles of one shape ahead of its requests."""
        n = self.lib.SRX_serverReserve(self.h, config, nx, ny, nimages, count)
        if n < count:
            raise SIReconError(_err(self.lib))
        return n

    def run_batch(self, items) -> None:
        """items: (config, raw, out) triples of any shapes (raw [nimages][ny][nx]
        uint16 or float32, out float32 of the result size, both C-contiguous).
        Blocks until every item's result is in its `out`."""
        arr = (BatchItem * len(items))()
        for i, (config, raw, out) in enumerate(items):
            if not raw.flags.c_contiguous or not out.flags.c_contiguous or out.dtype != np.float32:
                raise ValueError("raw and out must be C-contiguous, out float32")
            if raw.dtype not in (np.uint16, np.float32):
                raise ValueError("raw must be uint16 or float32")
            nimg, ny, nx = raw.shape
            arr[i] = BatchItem(config, nx, ny, nimg, raw.ctypes.data, int(raw.dtype == np.uint16), out.ctypes.data)
        if self.lib.SRX_serverRunBatch(self.h, arr, len(items)) != 0:
            raise SIReconError(_err(self.lib))

    def device_bytes(self) -> int:
        """Device bytes reserved against the budget (never above it)."""
        return int(self.lib.SRX_serverDeviceBytes(self.h))

    def planned_bytes(self, config: int, nx: int, ny: int, nimages: int) -> int:
        """Bytes admission reserves for a handle of this configuration and shape."""
        b = int(self.lib.SRX_serverPlannedBytes(self.h, config, nx, ny, nimages))
        if b == 0:
            raise SIReconError(_err(self.lib))
        return b

    def memory(self):
        """(reserved, held) device bytes, taken together."""
        r, h = C.c_size_t(0), C.c_size_t(0)
        self.lib.SRX_serverMemory(self.h, C.byref(r), C.byref(h))
        return r.value, h.value

    def device_bytes_held(self) -> int:
        """Device bytes the pooled handles actually hold now."""
        return int(self.lib.SRX_serverDeviceBytesHeld(self.h))

    def set_k0_reuse(self, config: int, on: bool = True) -> None:
        """Keep the first request's fitted k0 for the configuration's later
        requests (SRX_serverSetK0Reuse)."""
        if self.lib.SRX_serverSetK0Reuse(self.h, config, int(on)) != 0:
            raise SIReconError(_err(self.lib))

    def recorded_k0(self, config: int, ndirs: int = 3):
        k0 = np.zeros((ndirs, 2), np.float32)
        ok = self.lib.SRX_serverRecordedK0(self.h, config, k0.ctypes.data_as(C.POINTER(C.c_float)), ndirs)
        return k0 if ok else None

    def counters(self) -> dict:
        """Handles created, and deleted to stay within the budget, so far."""
        c, e = C.c_longlong(0), C.c_longlong(0)
        self.lib.SRX_serverCounters(self.h, C.byref(c), C.byref(e))
        return {"created": c.value, "evicted": e.value,
                "admission_waits": int(self.lib.SRX_serverAdmissionWaits(self.h))}

    def close(self):
        if self.h:
            self.lib.SRX_serverDestroy(self.h)
            self.h = None
        self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
