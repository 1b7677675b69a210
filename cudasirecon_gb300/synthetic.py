"""Seeded synthetic 3-beam SIM acquisitions and rotationally averaged OTFs.

Used to make workloads with the shapes of the reconstruction benchmarks (no
public dataset is involved).  The forward model is the standard 3-beam SIM
image formation with the illumination pattern moving with the focal plane:

    D_{d,p}(r) = [S * (1 + m2 cos(2 pi 2k_d.r + 2 phi_p))] (x) PSF
               + [S * m1 cos(2 pi k_d.r + phi_p)]          (x) (PSF * cos(2 pi kz1 z))

with k_d of magnitude 1/(2 ls) along the pattern angle of direction d,
phi_p = 2 pi p / nphases, kz1 = nimm/lambda_ex (1 - cos beta),
sin beta = lambda_ex / (2 ls nimm), lambda_ex = 0.88 lambda_em (the ratio
the reconstruction itself assumes).  The PSF is a scalar widefield pupil
integral; Poisson noise, a camera offset and uint16 clipping follow.

The scene is 100 nm beads (points at uniform random positions, lognormal
brightness) plus random-walk filaments.  Everything is float32 numpy/scipy;
no GPU is used.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

try:
    import scipy.fft as _fft

    def _fftn(a, axes=None):
        return _fft.fftn(a, axes=axes, workers=-1)

    def _ifftn(a, axes=None):
        return _fft.ifftn(a, axes=axes, workers=-1)
except Exception:  # pragma: no cover - scipy is present on both hosts
    _fftn = np.fft.fftn
    _ifftn = np.fft.ifftn


@dataclass
class Optics:
    na: float = 1.42
    nimm: float = 1.515
    wave_nm: float = 528.0
    ls: float = 0.2035
    dxy: float = 0.08
    dz: float = 0.125
    angles: tuple = (-0.8043, -1.8555, 0.2388)
    nphases: int = 5

    @property
    def lambda_em(self) -> float:
        return self.wave_nm / 1000.0

    @property
    def lambda_ex(self) -> float:
        return 0.88 * self.lambda_em

    def kz1(self) -> float:
        # axial frequency of the order-1 interference term (3-beam pattern)
        sinb = self.lambda_ex / (2.0 * self.ls * self.nimm)
        sinb = min(sinb, 0.999)
        return self.nimm / self.lambda_ex * (1.0 - math.sqrt(1.0 - sinb * sinb))


def widefield_psf(nx: int, ny: int, nz: int, optics: Optics) -> np.ndarray:
    """Scalar widefield PSF |pupil integral|^2 on an (nz, ny, nx) grid, peak-centred at (0,0,0) (FFT order), sum 1."""
    kx = np.fft.fftfreq(nx, d=optics.dxy)
    ky = np.fft.fftfreq(ny, d=optics.dxy)
    kr2 = ky[:, None] ** 2 + kx[None, :] ** 2
    kmax = optics.na / optics.lambda_em
    nk = optics.nimm / optics.lambda_em
    pupil = (kr2 <= kmax * kmax).astype(np.float64)
    kz = np.sqrt(np.maximum(nk * nk - kr2, 0.0))
    zs = (np.fft.fftfreq(nz, d=1.0 / nz)) * optics.dz  # signed z in FFT order
    psf = np.empty((nz, ny, nx), np.float64)
    for iz, z in enumerate(zs):
        amp = np.fft.ifft2(pupil * np.exp(2j * np.pi * kz * z))
        psf[iz] = np.abs(amp) ** 2
    psf /= psf.sum()
    return psf


def make_scene(nx: int, ny: int, nz: int, optics: Optics, rng: np.random.Generator,
               bead_density: float = 0.5, n_filaments: int = 50, drift_px: float = 0.0,
               bleach: float = 1.0) -> np.ndarray:
    """Point-like beads plus random-walk filaments deposited on the (nz, ny, nx) grid."""
    vol = np.zeros((nz, ny, nx), np.float32)
    lx, ly, lz = nx * optics.dxy, ny * optics.dxy, nz * optics.dz
    nbeads = int(bead_density * lx * ly * lz)
    pts = rng.uniform(0, 1, size=(nbeads, 3)) * np.array([nx, ny, nz])
    inten = rng.lognormal(0.0, 0.3, size=nbeads).astype(np.float32)
    xi = (np.floor(pts[:, 0] + drift_px).astype(np.int64)) % nx
    yi = np.floor(pts[:, 1]).astype(np.int64) % ny
    zi = np.floor(pts[:, 2]).astype(np.int64) % nz
    np.add.at(vol, (zi, yi, xi), inten)
    step = 0.05  # um
    persistence = 1.0  # um
    for _ in range(n_filaments):
        length = rng.uniform(5.0, 15.0)
        nsteps = int(length / step)
        pos = rng.uniform(0, 1, 3) * np.array([lx, ly, lz])
        d = rng.normal(size=3)
        d[2] *= 0.2
        d /= np.linalg.norm(d)
        sig = math.sqrt(2.0 * step / persistence)
        path = np.empty((nsteps, 3))
        for s in range(nsteps):
            d = d + rng.normal(scale=sig, size=3) * np.array([1, 1, 0.2])
            d /= np.linalg.norm(d)
            pos = pos + step * d
            path[s] = pos
        xi = (np.floor(path[:, 0] / optics.dxy + drift_px).astype(np.int64)) % nx
        yi = np.floor(path[:, 1] / optics.dxy).astype(np.int64) % ny
        zi = np.floor(path[:, 2] / optics.dz).astype(np.int64) % nz
        np.add.at(vol, (zi, yi, xi), np.float32(0.3))
    return vol * np.float32(bleach)


@dataclass
class Acquisition:
    raw: np.ndarray            # uint16 [ndirs*nz*nphases][ny][nx], Angle->Z->Phase order
    modamps: np.ndarray        # [ndirs][2] true m1, m2
    config: dict = field(default_factory=dict)


def simulate(nx: int, ny: int, nz: int, optics: Optics | None = None, seed: int = 1,
             peak_photons: float = 1000.0, background: float = 100.0, ndirs: int = 3,
             drift_px: float = 0.0, bleach: float = 1.0, scene_seed: int | None = None,
             mod_seed: int | None = None, noise_seed: int | None = None,
             n_filaments: int = 50, bead_density: float = 0.5) -> Acquisition:
    """Synthesise one SIM volume (3D when nz > 1, 2D otherwise)."""
    optics = optics or Optics()
    rs = np.random.default_rng(seed if scene_seed is None else scene_seed)
    rm = np.random.default_rng((seed + 1) if mod_seed is None else mod_seed)
    rn = np.random.default_rng((seed + 2) if noise_seed is None else noise_seed)
    scene = make_scene(nx, ny, nz, optics, rs, bead_density=bead_density, n_filaments=n_filaments,
                       drift_px=drift_px, bleach=bleach)
    psf = widefield_psf(nx, ny, nz, optics).astype(np.float32)
    zs = (np.fft.fftfreq(nz, d=1.0 / nz) * optics.dz).astype(np.float32)
    otf0 = _fftn(psf)
    if nz > 1:
        otf1 = _fftn(psf * np.cos(2 * np.pi * optics.kz1() * zs)[:, None, None])
    else:
        otf1 = otf0
    x = (np.arange(nx, dtype=np.float32) * optics.dxy)[None, None, :]
    y = (np.arange(ny, dtype=np.float32) * optics.dxy)[None, :, None]
    # 3D: order 1 at 1/(2 ls), order 2 at 1/ls; 2D (two-beam): order 1 at 1/ls
    k1 = 1.0 / (2.0 * optics.ls) if nz > 1 else 1.0 / optics.ls
    nph = optics.nphases
    m = np.stack([rm.uniform(0.5, 0.9, ndirs), rm.uniform(0.4, 0.8, ndirs)], axis=1)
    imgs = np.empty((ndirs, nz, nph, ny, nx), np.float32)
    for d in range(ndirs):
        th = optics.angles[d % len(optics.angles)]
        kx, ky = k1 * math.cos(th), k1 * math.sin(th)
        arg = 2 * np.pi * (kx * x + ky * y)
        for p in range(nph):
            phi = 2 * np.pi * p / nph
            if nz > 1:
                lat0 = 1.0 + m[d, 1] * np.cos(2 * arg + 2 * phi)
                lat1 = m[d, 0] * np.cos(arg + phi)
                img = np.real(_ifftn(_fftn(scene * lat0) * otf0 + _fftn(scene * lat1) * otf1))
            else:
                lat = 1.0 + m[d, 0] * np.cos(arg + phi)
                img = np.real(_ifftn(_fftn(scene * lat) * otf0))
            imgs[d, :, p] = img.astype(np.float32)
    imgs *= np.float32(peak_photons / max(float(imgs.max()), 1e-12))
    noisy = rn.poisson(np.maximum(imgs, 0)).astype(np.float32) + background
    raw = np.clip(np.rint(noisy), 0, 65535).astype(np.uint16)
    raw = raw.reshape(ndirs * nz * nph, ny, nx)
    return Acquisition(raw=raw, modamps=m)


def bead_psf_stack(nx: int, ny: int, nz: int, optics: Optics | None = None, nphases: int | None = None,
                   peak_photons: float = 1e5, background: float = 100.0, seed: int = 4,
                   offset_px: tuple = (0.3, -0.2, 0.15), pattern_phase: float = 0.3,
                   m1: float = 0.9, m2: float = 0.8) -> np.ndarray:
    """SIM PSF stack of one sub-resolution bead: the input of makeotf.

    float32 [nz * nphases][ny][nx], sections phase-fastest (section =
    z * nphases + phase).  The bead sits at the stack centre plus a
    sub-pixel offset (x, y, z in pixels) and the pattern moves with the
    focal plane, so with pattern phase phi0 at the bead the section at
    phase p is
      3D (nz > 1, 3-beam):  det0 (1 + m2 cos(2 phi_p + 2 phi0)) + m1 cos(phi_p + phi0) det1
      2D (nz = 1, 2-beam):  det0 (1 + m1 cos(phi_p + phi0))
    with det0 the widefield PSF at the bead and det1 the PSF times
    cos(2 pi kz1 (z - z_bead)).  Poisson noise on a constant background.
    """
    optics = optics or Optics()
    nph = nphases or optics.nphases
    rng = np.random.default_rng(seed)
    psf = widefield_psf(nx, ny, nz, optics).astype(np.float64)
    fx = np.fft.fftfreq(nx)[None, None, :]
    fy = np.fft.fftfreq(ny)[None, :, None]
    fz = np.fft.fftfreq(nz)[:, None, None]
    cz = (nz // 2 + offset_px[2]) if nz > 1 else 0.0
    shift = np.exp(-2j * np.pi * (fx * (nx // 2 + offset_px[0]) + fy * (ny // 2 + offset_px[1]) + fz * cz))
    det0 = np.real(np.fft.ifftn(np.fft.fftn(psf) * shift))
    stack = np.empty((nz, nph, ny, nx), np.float64)
    if nz > 1:
        zs = np.fft.fftfreq(nz, d=1.0 / nz) * optics.dz
        psf1 = psf * np.cos(2 * np.pi * optics.kz1() * zs)[:, None, None]
        det1 = np.real(np.fft.ifftn(np.fft.fftn(psf1) * shift))
        for p in range(nph):
            phi = 2 * np.pi * p / nph
            stack[:, p] = det0 * (1.0 + m2 * np.cos(2 * phi + 2 * pattern_phase)) + \
                m1 * np.cos(phi + pattern_phase) * det1
    else:
        for p in range(nph):
            phi = 2 * np.pi * p / nph
            stack[:, p] = det0 * (1.0 + m1 * np.cos(phi + pattern_phase))
    stack *= peak_photons / max(float(stack.max()), 1e-30)
    noisy = rng.poisson(np.maximum(stack, 0.0)).astype(np.float64) + background
    return noisy.reshape(nz * nph, ny, nx).astype(np.float32)


def ra_otf(optics: Optics, nx_psf: int = 128, nz_psf: int = 64, dz_psf: float | None = None,
           norders: int = 3, twod: bool = False) -> np.ndarray:
    """Rotationally averaged OTF pages in the layout of an OTF TIFF.

    3D: float32 [norders][nxotf = nx_psf/2+1][2*nz_psf]  (kr rows, complex kz along a row, FFT order).
    2D: float32 [norders][1][2*(nx_psf/2+1)]             (complex kr along the row).
    Bands are normalised by the order-0 DC value, as makeotf does.
    """
    dz_psf = dz_psf or optics.dz
    o = Optics(**{**optics.__dict__})
    o.dz = dz_psf
    nzp = 1 if twod else nz_psf
    psf = widefield_psf(nx_psf, nx_psf, nzp, o)
    zs = np.fft.fftfreq(nzp, d=1.0 / nzp) * dz_psf
    otfs = [np.fft.fftn(psf)]
    if not twod:
        otfs.append(np.fft.fftn(psf * np.cos(2 * np.pi * o.kz1() * zs)[:, None, None]))
        otfs.append(otfs[0])
    else:
        otfs.append(otfs[0])
    otfs = otfs[:norders]
    nr = nx_psf // 2 + 1
    kx = np.fft.fftfreq(nx_psf)
    kr = np.sqrt(kx[None, :] ** 2 + kx[:, None] ** 2) * nx_psf
    rbin = np.rint(kr).astype(np.int64)
    dc = otfs[0][0, 0, 0].real
    pages = []
    for ot in otfs:
        ra = np.zeros((nr, nzp), np.complex128)
        cnt = np.bincount(rbin.ravel(), minlength=nr)[:nr]
        for iz in range(nzp):
            re = np.bincount(rbin.ravel(), weights=ot[iz].real.ravel(), minlength=nr)[:nr]
            im = np.bincount(rbin.ravel(), weights=ot[iz].imag.ravel(), minlength=nr)[:nr]
            ra[:, iz] = (re + 1j * im) / np.maximum(cnt, 1)
        ra /= dc
        if twod:
            page = np.zeros((1, 2 * nr), np.float32)
            page[0, 0::2] = ra[:, 0].real
            page[0, 1::2] = ra[:, 0].imag
        else:
            page = np.zeros((nr, 2 * nzp), np.float32)
            page[:, 0::2] = ra.real
            page[:, 1::2] = ra.imag
        pages.append(page)
    return np.stack(pages)


def config_text(optics: Optics | None = None, twod: bool = False, extra: dict | None = None,
                otf_file: str | None = None, dz_psf: float | None = None) -> str:
    """The reference-style key=value config for a synthetic acquisition."""
    o = optics or Optics()
    kv = {
        "nimm": o.nimm, "background": 100, "wiener": 0.001,
        "k0angles": ",".join(f"{a:.6f}" for a in o.angles), "ls": o.ls,
        "ndirs": 3, "nphases": 3 if twod else 5, "na": o.na, "otfRA": 1,
        "xyres": o.dxy, "zres": o.dz, "zresPSF": dz_psf or o.dz,
        "wavelength": int(round(o.wave_nm)),
    }
    if not twod:
        kv["dampenOrder0"] = 1
    if otf_file:
        kv["otf-file"] = otf_file
    if extra:
        kv.update(extra)
    return "\n".join(f"{k}={v}" for k, v in kv.items()) + "\n"
