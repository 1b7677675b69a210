"""FP64 CPU oracle for the 3-beam SIM reconstruction path (test infrastructure).

A numpy restatement of the reference's reconstruction, function by function,
each citing the reference lines it follows (paths relative to the
scopetools/cudasirecon checkout).  Only ``tests/``, ``__graft_entry__.smoke``
and the ``cpu_baseline`` leg / reference arm of ``bench.py`` may use it; the
product never imports it.

Arithmetic is float64 throughout (numpy FFTs share cuFFT's unnormalised sign
conventions: forward e^{-i}, inverse e^{+i}).  The integer support cut-offs,
the k0 / angle search grids and the other scalars whose rounding steers the
control flow are formed in float32 exactly as the reference's host code does,
so the oracle follows the same search path as the reference.

Parity pin: ``tests/golden/*.npz`` hold outputs of the reference's own CUDA
kernels (run through ``oracle/ref_harness``) and ``tests/test_oracle_golden.py``
checks this module against them.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

f32 = np.float32
SPOTRATIO = 0.1            # cudaSireconImpl.h:51
K0_WARNING_THRESH = 0.05   # cudaSireconImpl.h:55


# --------------------------------------------------------------------------
# parameters: SetDefaultParams (cudaSirecon.cpp:16-72) overridden by the
# program_options defaults (cudaSirecon.cpp:913-1009); setParams 1011-1070.
# --------------------------------------------------------------------------
@dataclass
class Params:
    k0startangle: float = 1.648
    linespacing: float = 0.172
    na: float = 1.2
    nimm: float = 1.33
    ndirs: int = 3
    nphases: int = 5
    norders_output: int = 0
    norders: int = 0
    bTwolens: bool = False
    bFastSIM: bool = False
    bBessel: bool = False
    BesselNA: float = 0.144
    BesselLambdaEx: float = 0.488
    otfcutoff: float = 0.006
    zoomfact: float = 2.0
    z_zoom: int = 1
    explodefact: float = 1.0
    bFilteroverlaps: int = 1
    recalcarrays: int = 1
    napodize: int = 10
    forceamp: list = field(default_factory=lambda: [0.0])
    k0angles: list = field(default_factory=list)
    bSearchforvector: int = 1
    bUseTime0k0: int = 1
    apodizeoutput: int = 2
    apoGamma: float = 1.0
    bSuppress_singularities: int = 1
    suppression_radius: int = 10
    bDampenOrder0: bool = False
    bFitallphases: int = 1
    do_rescale: int = 1
    equalizez: bool = False
    equalizet: bool = False
    bNoKz0: bool = False
    wiener: float = 0.01
    bRadAvgOTF: bool = False
    bOneOTFperAngle: bool = False
    dzPSF: float = 0.15
    constbkgd: float = 0.0
    dxy: float = 0.1
    dz: float = 0.2
    wave: int = 530
    otffile: str = ""
    # model the reference's int-sized reads of bool flags (see effective_nokz0)
    reference_flag_bytes: bool = True
    # OTF geometry (determine_otf_dimensions)
    nxotf: int = 0
    nyotf: int = 0
    nzotf: int = 0
    dkzotf: float = 0.0
    dkrotf: float = 0.0


def effective_nokz0(p: "Params") -> bool:
    """The kz=0 exclusion the reference's kernels actually apply.

    makeoverlaps and filterbands copy ``bool bNoKz0`` into an int __constant__
    with cudaMemcpyToSymbol(..., sizeof(int)) (gpuFunctionsImpl.cu:564-565,
    1317-1318).  In ReconParams (cudaSireconImpl.h:143-144) bNoKz0 sits at
    byte 142, a padding byte at 143 and ``float wiener`` at 144, so the int
    the kernels test is bNoKz0 | pad << 8 | (low 16 bits of wiener) << 16:
    non-zero -- kz=0 excluded -- whenever the low half of wiener's bit
    pattern is non-zero (e.g. wiener=0.001, 0x3A83126F).  The padding byte is
    taken as zero (value-initialised parameters).
    """
    if not p.reference_flag_bytes:
        return bool(p.bNoKz0)
    bits = int(np.array([p.wiener], np.float32).view(np.uint32)[0])
    return bool(p.bNoKz0) or (bits & 0xFFFF) != 0


def _bool(v: str) -> bool:
    return v.strip().lower() in ("1", "true", "yes", "on", "")


def parse_config(text: str) -> Params:
    """key=value config text -> Params, with the reference's option semantics."""
    p = Params()
    for line in text.splitlines():
        line = line.split("#", 1)[0]
        if "=" not in line:
            continue
        k, v = (s.strip() for s in line.split("=", 1))
        fl = lambda: float(np.float32(float(v)))  # noqa: E731
        it = lambda: int(float(v))  # noqa: E731
        m = {
            "ndirs": ("ndirs", it), "nphases": ("nphases", it), "nordersout": ("norders_output", it),
            "angle0": ("k0startangle", fl), "ls": ("linespacing", fl), "na": ("na", fl),
            "nimm": ("nimm", fl), "wiener": ("wiener", fl), "otfcutoff": ("otfcutoff", fl),
            "zoomfact": ("zoomfact", fl), "zzoom": ("z_zoom", it), "background": ("constbkgd", fl),
            "otfRA": ("bRadAvgOTF", lambda: _bool(v)), "otfPerAngle": ("bOneOTFperAngle", lambda: _bool(v)),
            "fastSI": ("bFastSIM", lambda: _bool(v)), "k0searchAll": ("bUseTime0k0", it),
            "norescale": ("do_rescale", it), "equalizez": ("equalizez", lambda: _bool(v)),
            "equalizet": ("equalizet", lambda: _bool(v)), "dampenOrder0": ("bDampenOrder0", lambda: _bool(v)),
            "nosuppress": ("bSuppress_singularities", it), "nokz0": ("bNoKz0", lambda: _bool(v)),
            "gammaApo": ("apoGamma", fl), "explodefact": ("explodefact", fl),
            "nofilterovlps": ("bFilteroverlaps", lambda: int(_bool(v))), "bessel": ("bBessel", lambda: _bool(v)),
            "besselExWave": ("BesselLambdaEx", fl), "besselNA": ("BesselNA", fl),
            "xyres": ("dxy", fl), "zres": ("dz", fl), "zresPSF": ("dzPSF", fl),
            "wavelength": ("wave", it), "otf-file": ("otffile", lambda: v),
            "referenceFlagBytes": ("reference_flag_bytes", lambda: _bool(v)),
        }
        if k in m:
            name, conv = m[k]
            setattr(p, name, conv())
        elif k == "forcemodamp":
            p.forceamp = [float(np.float32(float(x))) for x in v.split()]
        elif k == "k0angles":
            p.k0angles = [float(np.float32(float(x))) for x in v.split(",") if x.strip()]
    return p


# --------------------------------------------------------------------------
# small helpers
# --------------------------------------------------------------------------
def makematrix(nphases: int, norders: int) -> np.ndarray:
    """Default branch of makematrix, cudaSirecon.cpp:606-617 (un-normalised)."""
    phi = 2.0 * math.pi / nphases
    m = np.zeros((2 * norders - 1, nphases))
    for j in range(nphases):
        m[0, j] = 1.0
        for o in range(1, norders):
            m[2 * o - 1, j] = math.cos(j * o * phi)
            m[2 * o, j] = math.sin(j * o * phi)
    return m


def otf_interp(otf: np.ndarray, kx, ky, kz, kzscale: float, nzotf: int, dkrotf: float):
    """dev_otfinterpolate for a rotationally averaged OTF, gpuFunctionsImpl.cu:1677-1715.

    ``otf`` is the flat complex array [nxotf*nzotf] (kr-major, kz fastest).
    """
    kx = np.asarray(kx, np.float64)
    ky = np.asarray(ky, np.float64)
    kz = np.broadcast_to(np.asarray(kz, np.float64), np.broadcast(kx, ky).shape)
    krindex = np.sqrt(kx * kx + ky * ky) / dkrotf
    kzindex = kz * kzscale
    kzindex = np.where(kzindex < 0, kzindex + nzotf, kzindex)
    ir = np.floor(krindex).astype(np.int64)
    iz = np.floor(kzindex).astype(np.int64)
    ar = krindex - ir
    az = kzindex - iz
    izp = np.where(iz == nzotf - 1, 0, iz + 1)
    n = otf.shape[0]
    def g(r, z):
        return otf[np.clip(r * nzotf + z, 0, n - 1)]
    v00 = g(ir, iz)
    v01 = g(ir, izp)
    v10 = g(ir + 1, iz)
    v11 = g(ir + 1, izp)
    return (1 - ar) * (v00 * (1 - az) + v01 * az) + ar * (v10 * (1 - az) + v11 * az)


def suppress(x):
    """dev_suppress, gpuFunctionsImpl.cu:1732-1739."""
    x6 = x * x * x
    x6 = x6 * x6
    return 1.0 / (1 + 20000 / (x6 + 20))


def order0damping(radius, zindex, rlimit, zlimit):
    """dev_order0damping, gpuFunctionsImpl.cu:1717-1725."""
    rf = radius / rlimit
    zf = np.abs(zindex / zlimit)
    return rf * rf + zf * zf * zf


def fitparabola(a1, a2, a3):
    """fitparabola, gpuFunctionsImpl.cu:479-495."""
    slope = 0.5 * (a3 - a1)
    curve = (a3 + a1) - 2 * a2
    if curve == 0:
        return 0.0
    peak = -slope / curve
    if peak > 1.5 or peak < -1.5:
        return 0.0
    return peak


def fitxyparabola(x1, y1, x2, y2, x3, y3):
    """fitxyparabola, gpuFunctionsImpl.cu:1022-1044 (float32 like the reference)."""
    x1, y1, x2, y2, x3, y3 = (f32(v) for v in (x1, y1, x2, y2, x3, y3))
    if x1 == x2 or x2 == x3 or x3 == x1:
        return f32(0.0)
    xbar1 = f32(0.5) * (x1 + x2)
    xbar2 = f32(0.5) * (x2 + x3)
    slope1 = (y2 - y1) / (x2 - x1)
    slope2 = (y3 - y2) / (x3 - x2)
    curve = (slope2 - slope1) / (xbar2 - xbar1)
    if curve == 0:
        return f32(0.0)
    return f32(xbar2 - slope2 / curve)


def findpeak(arr: np.ndarray):
    """findpeak, gpuFunctionsImpl.cu:443-477 (first maximum in row-major order)."""
    sizey, sizex = arr.shape
    flat = int(np.argmax(arr))
    ycent, xcent = divmod(flat, sizex)
    a1 = arr[ycent, (xcent - 1) % sizex]
    a2 = arr[ycent, xcent]
    a3 = arr[ycent, (xcent + 1) % sizex]
    px = fitparabola(a1, a2, a3) + xcent
    a1 = arr[(ycent - 1) % sizey, xcent]
    a3 = arr[(ycent + 1) % sizey, xcent]
    py = fitparabola(a1, a2, a3) + ycent
    return px, py


# --------------------------------------------------------------------------
# the reconstructor
# --------------------------------------------------------------------------
class SIMReconOracle:
    """Mirror of SIM_Reconstructor's in-memory flow (SR_new_from_shape path)."""

    def __init__(self, nx: int, ny: int, nimages: int, config: str | Params, otf_pages: np.ndarray):
        self.p = parse_config(config) if isinstance(config, str) else config
        p = self.p
        self.nx, self.ny = nx, ny
        # setup(), cudaSirecon.cpp:1104-1115
        self.nz = nimages // (p.nphases * p.ndirs)
        self.nz0 = self.nz
        self.ntimes = 1
        self.cur_time = 0
        # setup_common, cudaSirecon.cpp:1212-1217
        p.norders = p.norders_output if p.norders_output != 0 else p.nphases // 2 + 1
        self._setup_otf(np.asarray(otf_pages, np.float32))
        self.sep = makematrix(p.nphases, p.norders)
        self.noisevar = np.ones((p.ndirs, p.norders))
        # inscale, cudaSirecon.cpp:1231-1232
        self.inscale = f32(1.0 / (nx * ny * self.nz0 * p.zoomfact * p.zoomfact * p.z_zoom * p.ndirs))
        # k0guess, cudaSirecon.cpp:1236-1252
        k0mag = f32(1.0 / p.linespacing)
        if self.nz > 1:
            k0mag = f32(k0mag / f32(p.nphases // 2 + 1 - 1))
        delta = f32(math.pi / p.ndirs)
        self.k0guess = np.zeros((p.ndirs, 2))
        for i in range(p.ndirs):
            if len(p.k0angles) < p.ndirs:
                ang = f32(f32(p.k0startangle) + f32(i * delta))
            else:
                ang = f32(p.k0angles[i])
            self.k0guess[i] = [f32(k0mag * math.cos(ang)), f32(k0mag * math.sin(ang))]
        self.k0 = self.k0guess.copy()
        self.k0_time0 = np.zeros_like(self.k0)
        self.amp = np.zeros((p.ndirs, p.norders), np.complex128)
        self.amp[:, 0] = 1.0
        self.sum_dir0_phase0 = np.zeros(self.nz)
        self.planes = None
        self.bands = None
        self.result = None

    # determine_otf_dimensions (TIFF branch, cudaSirecon.cpp:1446-1482) +
    # loadOTFs (cudaSirecon.cpp:1540-1569)
    def _setup_otf(self, pages: np.ndarray):
        p = self.p
        nsec, h, w = pages.shape
        if self.nz == 1:
            p.nxotf, p.nyotf, p.nzotf = w // 2, (1 if p.bRadAvgOTF else h), 1
            p.dkrotf = float(f32(1 / (f32(p.dxy) * (w // 2 - 1) * 2)))
            p.dkzotf = 1.0
        elif p.bRadAvgOTF:
            p.nzotf, p.nxotf, p.nyotf = w // 2, h, 1
            p.dkzotf = float(f32(1 / (f32(p.dzPSF) * p.nzotf)))
            p.dkrotf = float(f32(1 / (f32(p.dxy) * (p.nxotf - 1) * 2)))
        else:
            raise NotImplementedError("only rotationally averaged OTFs are supported on the GPU path")
        size = p.nxotf * p.nyotf * p.nzotf
        cplx = pages.reshape(nsec, -1)[:, 0::2].astype(np.float64) + 1j * pages.reshape(nsec, -1)[:, 1::2]
        self.otf = []
        for i in range(p.norders):
            if nsec > i:
                self.otf.append(cplx[i, :size].copy())
            else:
                self.otf.append(cplx[0, :size].copy())

    # ---------------------------------------------------------------- load
    def set_raw(self, raw: np.ndarray):
        """setRaw -> loadImageData (cudaSirecon.cpp:1331-1435) + load_and_flatfield (1715-1731)."""
        p = self.p
        raw = np.asarray(raw).reshape(-1, self.ny, self.nx).astype(np.float64)
        planes = np.zeros((p.ndirs, p.nphases, self.nz, self.ny, self.nx))
        for d in range(p.ndirs):
            for z in range(self.nz):
                if p.bFastSIM:
                    zsec = z * p.ndirs * p.nphases + d * p.nphases
                else:
                    zsec = d * self.nz * p.nphases + z * p.nphases
                for ph in range(p.nphases):
                    planes[d, ph, z] = (raw[zsec + ph] - p.constbkgd - 0.0) * 1.0 * float(self.inscale)
        self.planes = planes

    def load_and_rescale(self, it: int):
        """rescaleDriver (cudaSirecon.cpp:520-540) -> rescale (gpuFunctionsImpl.cu:110-157)."""
        p = self.p
        if not p.do_rescale:
            return
        for d in range(p.ndirs):
            for z in range(self.nz):
                sums = self.planes[d, :, z].sum(axis=(1, 2))
                if d == 0 and not (p.equalizet and it != 0):
                    self.sum_dir0_phase0[z] = sums[0]
                ref = self.sum_dir0_phase0[0] if p.equalizez else self.sum_dir0_phase0[z]
                self.planes[d, :, z] *= (ref / sums)[:, None, None]

    def set_cur_time(self, it: int):
        self.cur_time = it

    # ------------------------------------------------------- band separation
    def apodize(self):
        """apodizationDriver (cudaSirecon.cpp:496-518) -> apodize_x/y_kernel (gpuFunctionsImpl.cu:52-82)."""
        n = self.p.napodize
        if n <= 0:
            return
        l = np.arange(n)
        fact = np.array([f32(1.0 - float(np.float32(math.sin(float(f32((li + 0.5) / f32(n) * math.pi * 0.5))))))
                         for li in l], np.float64)
        img = self.planes
        diff = (img[..., -1, :] - img[..., 0, :]) / 2.0
        for li in range(n):
            img[..., li, :] += diff * fact[li]
            img[..., self.ny - 1 - li, :] -= diff * fact[li]
        diff = (img[..., :, -1] - img[..., :, 0]) / 2.0
        for li in range(n):
            img[..., :, li] += diff * fact[li]
            img[..., :, self.nx - 1 - li] -= diff * fact[li]

    def separate_bands(self):
        """transformXYSlice (cudaSirecon.cpp:542-579), separate (gpuFunctionsImpl.cu:214-291), z FFT (cudaSirecon.cpp:238-257)."""
        p = self.p
        spec = np.fft.rfft2(self.planes, axes=(-2, -1))           # [dir][phase][z][ky][kx]
        bands = np.einsum("ij,djzyx->dizyx", self.sep, spec)       # [dir][band][z][ky][kx]
        if self.nz > 1:
            bands = np.fft.fft(bands, axis=2)
        self.bands = bands

    # ------------------------------------------------------------ overlaps
    def _scalars(self, k0x=0.0, k0y=0.0):
        p = self.p
        nx, ny, nz = self.nx, self.ny, self.nz0
        dxy = f32(p.dxy)
        dkx = f32(f32(1.0) / (nx * dxy))
        dky = f32(f32(1.0) / (ny * dxy))
        dkz = f32(f32(1.0) / (nz * f32(p.dz))) if p.dz > 0 else f32(p.dkzotf)
        kzscale = f32(dkz / f32(p.dkzotf))
        # float rdistcutoff = na*2.0/(wave*0.001), clamped to 1/(2 dxy): gpuFunctionsImpl.cu:518-519
        rdistcutoff = f32(float(f32(p.na)) * 2.0 / (p.wave * 0.001))
        if float(rdistcutoff) > 1.0 / (2.0 * float(dxy)):
            rdistcutoff = f32(1.0 / (2.0 * float(dxy)))
        lambdaem = f32((f32(p.wave) / f32(p.nimm)) / 1.0e3)
        lambdaexc = f32(0.88 * lambdaem)
        alpha = f32(math.asin(float(f32(f32(p.na) / f32(p.nimm)))))
        return dict(dkx=dkx, dky=dky, dkz=dkz, kzscale=kzscale, rdistcutoff=rdistcutoff,
                    lambdaem=lambdaem, lambdaexc=lambdaexc, alpha=alpha)

    def _zdist_overlaps(self, s):
        """zdistcutoff of makeoverlaps, gpuFunctionsImpl.cu:529-548."""
        zd = float(math.ceil(((1.0 - float(f32(math.cos(float(s["alpha"]))))) / float(s["lambdaem"])) / float(s["dkz"])))
        if zd > self.nz0 // 2:
            zd = float(max(self.nz0 // 2 - 1, 0))
        return int(zd)

    def makeoverlaps(self, d: int, order1: int, order2: int, k0x: float, k0y: float):
        """makeoverlaps (gpuFunctionsImpl.cu:497-675) with makeOverlaps0/1Kernel (677-872) and the inverse 3D/2D FFT."""
        p = self.p
        nx, ny, nz = self.nx, self.ny, self.nz0
        bands = self.bands[d]
        s = self._scalars()
        f02 = (4.0 if p.bBessel else 5.0) if nz > 1 else 1.0
        zdc = self._zdist_overlaps(s)
        kx = float(f32(f32(k0x) * (order2 - order1)))
        ky = float(f32(f32(k0y) * (order2 - order1)))
        otfcutoff = 0.01 if p.bBessel else p.otfcutoff
        cut = float(s["rdistcutoff"])
        j = np.arange(nx)
        i = np.arange(ny)
        x1f = np.where(j > nx // 2, j - nx, j) * float(s["dkx"])
        y1f = np.where(i > ny // 2, i - ny, i) * float(s["dky"])
        X1, Y1 = np.meshgrid(x1f, y1f)                   # [ny][nx]
        J, I = np.meshgrid(j, i)
        conj = J > nx // 2
        jin = np.where(conj, nx - J, J)
        iin = np.where(conj, (ny - I) % ny, I)
        rdist1 = np.sqrt(X1 * X1 + Y1 * Y1)
        x12, y12 = X1 - kx, Y1 - ky
        x21, y21 = X1 + kx, Y1 + ky
        rdist12 = np.sqrt(x12 * x12 + y12 * y12)
        rdist21 = np.sqrt(x21 * x21 + y21 * y21)
        ov0 = np.zeros((nz, ny, nx), np.complex128)
        ov1 = np.zeros((nz, ny, nx), np.complex128)
        b1re = bands[0] if order1 == 0 else bands[2 * order1 - 1]
        b1im = None if order1 == 0 else bands[2 * order1]
        b2re, b2im = bands[2 * order2 - 1], bands[2 * order2]
        otf_1, otf_2 = self.otf[order1], self.otf[order2]
        kzs, nzo, dkr = float(s["kzscale"]), p.nzotf, p.dkrotf
        for z0 in range(-zdc, zdc + 1):
            if z0 == 0 and effective_nokz0(p):
                continue
            zin = np.where(conj, (-z0 + nz) % nz, (z0 + nz) % nz)
            zout = (z0 + nz) % nz
            # overlap 0 (order1 band, weighted by the order2 OTF)
            m0 = (rdist1 <= cut) & (rdist12 <= cut)
            o1 = otf_interp(otf_1, X1, Y1, z0, kzs, nzo, dkr)
            o12 = otf_interp(otf_2, x12, y12, z0, kzs, nzo, dkr)
            m0 &= (np.abs(o1) > otfcutoff) & (np.abs(o12) * f02 > otfcutoff)
            root = np.sqrt(np.abs(o1) ** 2 + np.abs(o12) ** 2)
            fact = np.where(m0, o12 / np.where(root > 0, root, 1), 0)
            v1re = b1re[zin, iin, jin]
            v1im = b1im[zin, iin, jin] if b1im is not None else 0 * v1re
            v1re = np.where(conj, np.conj(v1re), v1re) * fact
            v1im = np.where(conj, np.conj(v1im), v1im) * fact
            ov0[zout] = np.where(m0, v1re + 1j * v1im, 0)
            # overlap 1 (order2 band, weighted by the order1 OTF)
            m1 = (rdist1 < cut) & (rdist21 <= cut)
            o2 = otf_interp(otf_2, X1, Y1, z0, kzs, nzo, dkr)
            o21 = otf_interp(otf_1, x21, y21, z0, kzs, nzo, dkr)
            m1 &= (np.abs(o2) * f02 > otfcutoff) & (np.abs(o21) > otfcutoff)
            root = np.sqrt(np.abs(o2) ** 2 + np.abs(o21) ** 2)
            fact = np.where(m1, o21 / np.where(root > 0, root, 1), 0)
            v2re = np.where(conj, np.conj(b2re[zin, iin, jin]), b2re[zin, iin, jin]) * fact
            v2im = np.where(conj, np.conj(b2im[zin, iin, jin]), b2im[zin, iin, jin]) * fact
            ov1[zout] = np.where(m1, v2re + 1j * v2im, 0)
        n = nx * ny * nz
        axes = (0, 1, 2) if nz > 1 else (1, 2)
        scale = n if nz > 1 else nx * ny
        self.overlap0 = np.fft.ifftn(ov0, axes=axes) * scale
        self.overlap1 = np.fft.ifftn(ov1, axes=axes) * scale
        return self.overlap0, self.overlap1

    def findrealspacemodamp(self, d, order1, order2, k0x, k0y, redoarrays):
        """findrealspacemodamp + reductionKernel, gpuFunctionsImpl.cu:1074-1220."""
        if redoarrays:
            self.makeoverlaps(d, order1, order2, k0x, k0y)
        nx, ny = self.nx, self.ny
        kx = float(f32(f32(k0x) * (order2 - order1)))
        ky = float(f32(f32(k0y) * (order2 - order1)))
        X, Y = self.overlap0, self.overlap1
        xsy = (np.conj(X) * Y).sum(axis=0)                     # [ny][nx]
        ii = np.arange(nx)[None, :] - 0.5 * nx
        jj = np.arange(ny)[:, None] - 0.5 * ny
        ang = 2.0 * math.pi * (ii * kx + jj * ky) * float(f32(self.p.dxy))
        xstary = (xsy * np.exp(1j * ang)).sum()
        sx = (np.abs(X) ** 2).sum()
        sy = (np.abs(Y) ** 2).sum()
        m1 = xstary / sx
        m2 = np.conj(xstary) / sy
        tan2beta = 2.0 * abs(xstary) / (sx - sy)
        beta = 0.5 * math.atan(tan2beta)
        if beta < 0:
            beta += 0.5 * math.pi
        m3 = math.tan(beta) * np.exp(1j * np.angle(xstary))
        corr = math.sqrt(abs(xstary) ** 2 / (sx * sy))
        return m1, m2, m3, corr

    def getmodamp(self, d, kangle, klength, order1, order2, redoarrays):
        """getmodamp, gpuFunctionsImpl.cu:1046-1072."""
        k1x = float(f32(f32(klength) * f32(math.cos(float(f32(kangle))))))
        k1y = float(f32(f32(klength) * f32(math.sin(float(f32(kangle))))))
        m1, _, _, _ = self.findrealspacemodamp(d, order1, order2, k1x, k1y, redoarrays)
        return f32(m1.real * m1.real + m1.imag * m1.imag), m1

    def findk0(self, d):
        """findk0, gpuFunctionsImpl.cu:306-372."""
        p = self.p
        nx, ny, nz = self.nx, self.ny, self.nz0
        fitorder2 = (1 if p.bBessel else 2) if nz > 1 else 1
        k0 = self.k0[d]
        X, Y = self.makeoverlaps(d, 0, fitorder2, k0[0], k0[1])
        cc = (X * np.conj(Y)).sum(axis=0)
        inten = np.abs(np.fft.fft2(cc)) ** 2
        px, py = findpeak(inten)
        dxy = float(f32(p.dxy))
        dkx = float(f32(1 / (nx * f32(dxy))))
        dky = float(f32(1 / (ny * f32(dxy))))
        if k0[0] / dkx < px - nx // 2:
            px -= nx
        if k0[0] / dkx > px + nx // 2:
            px += nx
        if k0[1] / dky < py - ny // 2:
            py -= ny
        if k0[1] / dky > py + ny // 2:
            py += ny
        self.k0[d] = [float(f32(px * dkx / fitorder2)), float(f32(py * dky / fitorder2))]

    def fitk0andmodamps(self, d):
        """fitk0andmodamps, gpuFunctionsImpl.cu:874-1020 (same float32 search grid)."""
        p = self.p
        nx, ny, nz = self.nx, self.ny, self.nz0
        fitorder1 = 0
        fitorder2 = (1 if p.bBessel else 2) if nz > 1 else 1
        k0 = self.k0[d]
        k0mag = f32(math.sqrt(float(f32(k0[0])) ** 2 + float(f32(k0[1])) ** 2))
        k0angle = f32(math.atan2(float(f32(k0[1])), float(f32(k0[0]))))
        redo = int(p.recalcarrays >= 1)
        x2 = k0angle
        amp2, _ = self.getmodamp(d, k0angle, k0mag, fitorder1, fitorder2, redo)
        redo = int(p.recalcarrays >= 3)
        dang = f32(0.001)
        dmag = f32(0.1 / (max(nx, ny) * float(f32(p.dxy))))
        angle = f32(k0angle + dang)
        x3 = angle
        amp3, _ = self.getmodamp(d, angle, k0mag, fitorder1, fitorder2, redo)
        amp1 = f32(0)
        x1 = f32(0)
        if amp3 > amp2:
            while amp3 > amp2:
                amp1, x1, amp2, x2 = amp2, x2, amp3, x3
                angle = f32(angle + dang)
                x3 = angle
                amp3, _ = self.getmodamp(d, angle, k0mag, fitorder1, fitorder2, redo)
        else:
            angle = k0angle
            amp3, amp2 = amp2, amp3
            x3, x2 = x2, x3
            while amp3 > amp2:
                amp1, x1, amp2, x2 = amp2, x2, amp3, x3
                angle = f32(angle - dang)
                x3 = angle
                amp3, _ = self.getmodamp(d, angle, k0mag, fitorder1, fitorder2, redo)
        angle = fitxyparabola(x1, amp1, x2, amp2, x3, amp3)
        x2 = k0mag
        amp2, _ = self.getmodamp(d, angle, k0mag, fitorder1, fitorder2, redo)
        mag = f32(k0mag + dmag)
        x3 = mag
        amp3, _ = self.getmodamp(d, angle, mag, fitorder1, fitorder2, redo)
        if amp3 > amp2:
            while amp3 > amp2:
                amp1, x1, amp2, x2 = amp2, x2, amp3, x3
                mag = f32(mag + dmag)
                x3 = mag
                amp3, _ = self.getmodamp(d, angle, mag, fitorder1, fitorder2, redo)
        else:
            mag = k0mag
            amp3, amp2 = amp2, amp3
            x3, x2 = x2, x3
            while amp3 > amp2:
                amp1, x1, amp2, x2 = amp2, x2, amp3, x3
                mag = f32(mag - dmag)
                x3 = mag
                amp3, _ = self.getmodamp(d, angle, mag, fitorder1, fitorder2, redo)
        mag = fitxyparabola(x1, amp1, x2, amp2, x3, amp3)
        redo = int(p.recalcarrays >= 2)
        _, modamp = self.getmodamp(d, angle, mag, fitorder1, fitorder2, redo)
        self.k0[d] = [float(f32(mag * f32(math.cos(float(angle))))), float(f32(mag * f32(math.sin(float(angle)))))]
        self.amp[d, fitorder2] = modamp
        if nz == 1:
            for order in range(2, p.norders):
                _, m = self.getmodamp(d, angle, mag, order - 1, order, 1)
                self.amp[d, order] = m
        else:
            for order in range(1, p.norders):
                if order != fitorder2:
                    _, m = self.getmodamp(d, angle, mag, 0, order, 1)
                    self.amp[d, order] = m

    def fit(self):
        """k0/modamp part of findModulationVectorsAndPhasesForAllDirections, cudaSirecon.cpp:296-493."""
        p = self.p
        reuse = self.ntimes > 1 and self.cur_time > 0 and p.bUseTime0k0
        for d in range(p.ndirs):
            if not reuse:
                self.k0[d] = self.k0guess[d]
            if p.bSearchforvector and not reuse:
                self.findk0(d)
                p.recalcarrays = 1
                self.fitk0andmodamps(d)
                if self.cur_time == 0:
                    self.k0_time0[d] = self.k0[d]
                dist = math.hypot(self.k0[d][0] - self.k0guess[d][0], self.k0[d][1] - self.k0guess[d][1])
                if self.ntimes > 1 and self.cur_time > 0 and dist > 2 * K0_WARNING_THRESH:
                    self.k0[d] = self.k0_time0[d]
                    for order in range(1, p.norders):
                        o1 = 0 if self.nz0 > 1 else order - 1
                        m1, _, _, _ = self.findrealspacemodamp(d, o1, order, *self.k0[d], 1)
                        self.amp[d, order] = m1
            else:
                for order in range(1, p.norders):
                    m1, _, _, _ = self.findrealspacemodamp(d, 0, order, *self.k0[d], 1)
                    self.amp[d, order] = m1
            if self.nz == 1:
                for order in range(2, p.norders):
                    self.amp[d, order] = self.amp[d, order] * self.amp[d, order - 1]
            if p.forceamp[0] > 0.0:
                for order in range(1, p.norders):
                    a = abs(self.amp[d, order])
                    if a < p.forceamp[order - 1]:
                        self.amp[d, order] *= p.forceamp[order - 1] / a
            if not p.bFitallphases:
                base = np.angle(self.amp[d, 1])
                for order in range(2, p.norders):
                    self.amp[d, order] = abs(self.amp[d, order]) * np.exp(1j * order * base)

    # ------------------------------------------------------------- filter
    def filter_cutoffs(self):
        """zdistcutoff / apocutoff of filterbands, gpuFunctionsImpl.cu:1241-1298 (single-lens, non-Bessel)."""
        p = self.p
        s = self._scalars()
        no = p.norders
        zdc = [0] * no
        # evaluated in float: (int) ceil(((1-cosf(alpha))/lambdaem) / dkz), gpuFunctionsImpl.cu:1254
        t = f32(f32(f32(1.0) - f32(math.cos(float(s["alpha"])))) / s["lambdaem"])
        zdc[0] = int(math.ceil(float(f32(t / s["dkz"]))))
        zdc[no - 1] = int(1.3 * zdc[0])
        if no >= 3:
            for o in range(1, no - 1):
                zdc[o] = int(f32(f32(1) + f32(s["lambdaem"] / s["lambdaexc"])) * f32(zdc[0]))
        for o in range(no):
            if zdc[o] >= self.nz0 // 2:
                zdc[o] = max(self.nz0 // 2 - 1, 0)
        return zdc, s

    def filterbands(self, d):
        """filterbands (gpuFunctionsImpl.cu:1222-1441), kernel1 twice per order then kernel3 (1443-1675)."""
        p = self.p
        nx, ny, nz = self.nx, self.ny, self.nz0
        no = p.norders
        zdc, s = self.filter_cutoffs()
        wiener = float(f32(p.wiener) * f32(p.wiener))
        k0 = self.k0
        k0mag = float(f32(math.sqrt(float(f32(k0[0][0])) ** 2 + float(f32(k0[0][1])) ** 2)))
        cut = float(s["rdistcutoff"])
        apocutoff = cut + k0mag * (no - 1)
        zapocutoff = zdc[1] if no > 1 else 0
        ampmag2 = np.abs(self.amp) ** 2
        conjamp = np.conj(self.amp[d])
        # filterbands_kernel1 forms coordinates and radii in float32
        # (gpuFunctionsImpl.cu:1456-1505); the support / suppression tests
        # below are decided on those float32 values.
        dkx = f32(1.0 / (nx * float(f32(p.dxy))))
        dky = f32(1.0 / (ny * float(f32(p.dxy))))
        min_dkr = min(dkx, dky)
        supp_r = f32(p.suppression_radius) * min_dkr
        cut = f32(cut)
        k0 = np.asarray(k0, np.float64).astype(f32)
        kzs, nzo, dkr = float(s["kzscale"]), p.nzotf, p.dkrotf
        nv = self.noisevar
        nokz0 = effective_nokz0(p)
        B = self.bands[d]
        nxh = nx // 2 + 1
        for order in range(no):
            kx, ky = f32(order) * k0[d][0], f32(order) * k0[d][1]
            b1 = B[0] if order == 0 else B[2 * order - 1]
            b2 = None if order == 0 else B[2 * order]
            for second in (False, True):
                x1 = np.arange(1, nx // 2 + 1)
                if second:
                    x1 = x1 - nx // 2
                y1 = np.arange(-(ny // 2), ny - ny // 2)
                z0 = np.arange(-zdc[order], zdc[order] + 1)
                Z0, Y1, X1 = np.meshgrid(z0, y1, x1, indexing="ij")
                conj = X1 < 0
                iin = np.where(conj, -Y1, Y1)
                jin = np.where(conj, -X1, X1)
                keep = ~(conj & (order == 0))
                iin = np.where(iin < 0, iin + ny, iin)
                x1f = X1.astype(f32) * dkx
                y1f = Y1.astype(f32) * dky
                rdist1 = np.sqrt(x1f * x1f + y1f * y1f)
                insup = (rdist1 <= cut) & keep
                outsup = (rdist1 > cut) & keep
                # out-of-support zeroing uses z0 (not the conj-flipped z): gpuFunctionsImpl.cu:1647-1652
                izo = (Z0[outsup] + nz) % nz
                b1[izo, iin[outsup], jin[outsup]] = 0
                if b2 is not None:
                    b2[izo, iin[outsup], jin[outsup]] = 0
                X1s, Y1s, Z0s = x1f[insup], y1f[insup], Z0[insup]
                r1 = rdist1[insup]
                cj = conj[insup]
                xabs, yabs = X1s + kx, Y1s + ky
                rabs = np.sqrt(xabs * xabs + yabs * yabs)
                o1 = otf_interp(self.otf[order], X1s, Y1s, Z0s, kzs, nzo, dkr)
                weight = np.abs(o1) ** 2
                if order != 0:
                    weight = weight * ampmag2[d, order]
                damp = np.full(r1.shape, 1.0 / nv[d, order])
                if p.bSuppress_singularities and order != 0:
                    damp = np.where(r1 <= supp_r, damp * suppress(r1 / min_dkr), damp)
                elif (not p.bDampenOrder0) and p.bSuppress_singularities and order == 0:
                    damp = np.where(r1 <= supp_r, damp * suppress(r1 / min_dkr), damp)
                elif p.bDampenOrder0 and order == 0:
                    damp = damp * order0damping(r1, Z0s, cut, zdc[0])
                if order == 0 and nokz0:
                    damp = np.where(Z0s == 0, 0.0, damp)
                sumw = weight * damp
                for d2 in range(p.ndirs):
                    for o2 in range(-(no - 1), no):
                        if d2 == d and o2 == order:
                            continue
                        if not p.bFilteroverlaps and not (o2 == 0 and order == 0):
                            continue
                        a2 = abs(o2)
                        x2 = xabs - f32(o2) * k0[d2][0]
                        y2 = yabs - f32(o2) * k0[d2][1]
                        r2 = np.sqrt(x2 * x2 + y2 * y2)
                        m = r2 < cut
                        o2v = otf_interp(self.otf[a2], x2, y2, Z0s, kzs, nzo, dkr)
                        w = np.abs(o2v) ** 2 / nv[d2, a2]
                        if o2 != 0:
                            w = w * ampmag2[d2, a2]
                        if p.bSuppress_singularities and o2 != 0:
                            w = np.where(r2 <= supp_r, w * suppress(r2 / min_dkr), w)
                        elif (not p.bDampenOrder0) and p.bSuppress_singularities and o2 == 0:
                            w = np.where(r2 <= supp_r, w * suppress(r2 / min_dkr), w)
                        elif p.bDampenOrder0 and o2 == 0:
                            w = w * order0damping(r2, Z0s, cut, zdc[0])
                        if nokz0 and o2 == 0:
                            w = np.where(Z0s == 0, 0.0, w)
                        sumw = sumw + np.where(m, w, 0.0)
                sumw = sumw + wiener
                scale = damp * np.conj(o1) / sumw
                if p.apodizeoutput:
                    zabs = np.abs(Z0s)
                    if zapocutoff > 0:
                        rho = np.sqrt((rabs / apocutoff) ** 2 + (zabs / zapocutoff) ** 2)
                    else:
                        rho = np.sqrt((rabs / apocutoff) ** 2)
                    rho = np.minimum(rho, 1.0)
                    apo = np.cos(0.5 * math.pi * rho) if p.apodizeoutput == 1 else 1.0 - rho
                    scale = scale * apo
                zz = np.where(cj, -Z0s, Z0s)
                iz = (zz + nz) % nz
                ii, jj = iin[insup], jin[insup]
                if order == 0:
                    b1[iz, ii, jj] = b1[iz, ii, jj] * scale
                else:
                    scale = scale * conjamp[order]
                    re = b1[iz, ii, jj]
                    im = b2[iz, ii, jj]
                    re = np.where(cj, np.conj(re), re)
                    im = np.where(cj, np.conj(im), im)
                    plus = re + 1j * im
                    minus = re - 1j * im
                    plus = plus * scale
                    re = 0.5 * (plus + minus)
                    im = (plus - minus) / 2j
                    re = np.where(cj, np.conj(re), re)
                    im = np.where(cj, np.conj(im), im)
                    b1[iz, ii, jj] = re
                    b2[iz, ii, jj] = im
            # kernel3: clear planes outside +-zdistcutoff
            lo, hi = zdc[order] + 1, nz - zdc[order]
            if hi > lo:
                b1[lo:hi] = 0
                if b2 is not None:
                    b2[lo:hi] = 0

    # ------------------------------------------------------------ assembly
    def assemble(self, d, out):
        """assemblerealspacebands with move_kernel, cos_sin_kernel and write_outbuffer_kernel1/2, gpuFunctionsImpl.cu:1741-1954."""
        p = self.p
        nx, ny, nz = self.nx, self.ny, self.nz0
        X = int(round(p.zoomfact * nx))
        Y = int(round(p.zoomfact * ny))
        Z = p.z_zoom * nz
        B = self.bands[d]
        xs = np.arange(nx) - (nx // 2 - 1)
        ys = np.arange(ny) - (ny // 2 - 1)
        zs = (np.arange(nz) - (nz // 2 - 1)) if nz > 1 else np.zeros(1, np.int64)
        Zg, Yg, Xg = np.meshgrid(zs, ys, xs, indexing="ij")
        conj = Xg < 0
        xi = np.where(conj, -Xg, Xg)
        yi = np.where(conj, -Yg, Yg) % ny
        zi = np.where(conj, -Zg, Zg) % nz
        xo, yo, zo = Xg % X, Yg % Y, Zg % Z
        fact = p.explodefact / 0.5
        jx = np.arange(X) - X // 2
        iy = np.arange(Y) - Y // 2
        for order in range(p.norders):
            big = np.zeros((Z, Y, X), np.complex128)
            if order == 0:
                v = B[0][zi, yi, xi]
                v = np.where(conj, np.conj(v), v)
            else:
                re = B[2 * order - 1][zi, yi, xi]
                im = B[2 * order][zi, yi, xi]
                re = np.where(conj, np.conj(re), re)
                im = np.where(conj, np.conj(im), im)
                v = re + 1j * im
            big[zo, yo, xo] = v
            axes = (0, 1, 2) if Z > 1 else (1, 2)
            g = np.fft.ifftn(big, axes=axes) * (np.prod([big.shape[a] for a in axes]))
            if order == 0:
                out += g.real
            else:
                k0x = float(f32(k0c(self.k0[d][0]) * order))
                k0y = float(f32(k0c(self.k0[d][1]) * order))
                ang = fact * math.pi * (jx[None, :] * k0x + iy[:, None] * k0y) * (float(f32(p.dxy)) / p.zoomfact)
                out += 2.0 * (g.real * np.cos(ang) - g.imag * np.sin(ang))

    def process(self):
        """processOneVolume, cudaSirecon.cpp:1264-1321."""
        self.apodize()
        self.separate_bands()
        self.fit()
        p = self.p
        X = int(round(p.zoomfact * self.nx))
        Y = int(round(p.zoomfact * self.ny))
        out = np.zeros((p.z_zoom * self.nz0, Y, X))
        for d in range(p.ndirs):
            self.filterbands(d)
            self.assemble(d, out)
        self.result = out
        return 1


def k0c(v):
    return f32(v)
