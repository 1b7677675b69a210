"""CPU restatement of the reference's makeotf (src/otf/radialft.cpp): PSF
stack of a bead -> rotationally averaged SIM OTF.

TEST INFRASTRUCTURE ONLY.  The product computes this on the GPU
(cudasirecon_gb300/csrc/makeotf.cu); this module is the checker that the
tests, the fixture generator and the bench's CPU baseline use.  It is
pinned against the reference program itself (oracle/makeotf_ref.py runs
radialft.cpp compiled unmodified), see tests/test_makeotf_oracle.py.

Numerics follow the reference where its float32 arithmetic makes a decision
or is visible at the tolerance the tests use: apodisation, the phase-average
used to find the bead, the parabolic sub-pixel fits, the separation matrix,
the shift phases and the radial bin index (rint of a float32 quotient) are
float32 as in the reference, and so are the radial bin sums (in the
reference's order); the 3D FFT is float64 (the reference uses float32
FFTW).

Reference line numbers are of src/otf/radialft.cpp.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

f32 = np.float32


@dataclass
class MakeOTFOptions:
    """The switches of radialft.cpp:commandline (1381-1553) with their
    defaults from main (82-108)."""
    nphases: int = 5
    angle: float = 1.57          # -angle
    ls: float = 0.2              # -ls
    dr: float = 0.106            # -xyres
    dz: float = 0.1              # -zres
    beaddiam: float = 0.12       # -beaddiam
    na: float = 1.4              # -na
    nimm: float = 1.515          # -nimm
    wavelength: int = 525        # -wavelength
    background: float = -1.0     # -background (< 0: estimate from the border)
    fixorigin: tuple = (0, 0)    # -fixorigin kr1 kr2 (kr1 > 0 enables)
    leavekz: tuple = (0, 0, 0)   # -leavekz (first > 0 enables cleanup)
    ifixz: int = 1               # -ifixkz
    ifixr: int = 0               # -ifixkr
    rescale: bool = False        # -rescale
    five_bands: bool = False     # -5bands
    conj: bool = False           # -conj
    compensate: bool = True      # -nocompen clears it
    pishift: bool = False        # -PIshift
    bessel: bool = False         # -bessel

    @classmethod
    def from_args(cls, args: list[str]) -> "MakeOTFOptions":
        """Parse reference-style switches (no file names)."""
        o = cls()
        i = 0
        while i < len(args):
            a = args[i]
            nxt = args[i + 1] if i + 1 < len(args) else None
            if a == "-angle": o.angle = float(nxt); i += 2
            elif a == "-ls": o.ls = float(nxt); i += 2
            elif a == "-fixorigin": o.fixorigin = (int(args[i + 1]), int(args[i + 2])); i += 3
            elif a == "-leavekz": o.leavekz = (int(args[i + 1]), int(args[i + 2]), int(args[i + 3])); i += 4
            elif a == "-rescale": o.rescale = True; i += 1
            elif a == "-5bands": o.five_bands = True; i += 1
            elif a == "-conj": o.conj = True; i += 1
            elif a == "-nocompen": o.compensate = False; i += 1
            elif a == "-nphases": o.nphases = int(nxt); i += 2
            elif a == "-beaddiam": o.beaddiam = float(nxt); i += 2
            elif a == "-background": o.background = float(nxt); i += 2
            elif a == "-na": o.na = float(nxt); i += 2
            elif a == "-nimm": o.nimm = float(nxt); i += 2
            elif a == "-ifixkz": o.ifixz = int(nxt); i += 2
            elif a == "-ifixkr": o.ifixr = int(nxt); i += 2
            elif a == "-wavelength": o.wavelength = int(nxt); i += 2
            elif a == "-xyres": o.dr = float(nxt); i += 2
            elif a == "-zres": o.dz = float(nxt); i += 2
            elif a == "-bessel": o.bessel = True; i += 1
            elif a == "-PIshift": o.pishift = True; i += 1
            else:
                raise ValueError(f"unsupported makeotf switch {a!r}")
        return o


def estimate_background(sec: np.ndarray, border: int = 20) -> np.float32:
    """radialft.cpp:487-503: mean of the pixels with y < b, y > ny-b, x < b or
    x > nx-b (double sum)."""
    ny, nx = sec.shape
    y = np.arange(ny)[:, None]
    x = np.arange(nx)[None, :]
    m = (y < border) | (y > ny - border) | (x < border) | (x > nx - border)
    return f32(np.sum(sec[m].astype(np.float64)) / np.count_nonzero(m))


def apodize(img: np.ndarray, napodize: int = 10) -> None:
    """radialft.cpp:695-720, in place on a float32 [ny][nx] section: columns
    first, then rows (the rows use the column-blended ends)."""
    ny, nx = img.shape
    fact = np.array([f32(1.0 - math.sin(((float(f32(l)) + 0.5) / napodize) * math.pi * 0.5))
                     for l in range(napodize)], np.float32)
    diff = ((img[ny - 1, :] - img[0, :]) / f32(2)).astype(np.float32)
    for l in range(napodize):
        img[l, :] += diff * fact[l]
        img[ny - 1 - l, :] -= diff * fact[l]
    diff = ((img[:, nx - 1] - img[:, 0]) / f32(2)).astype(np.float32)
    for k in range(napodize):
        img[:, k] += diff * fact[k]
        img[:, nx - 1 - k] -= diff * fact[k]


def fitparabola(a1, a2, a3) -> np.float32:
    """radialft.cpp:672-690 (float32): vertex offset of the parabola through
    (-1,a1), (0,a2), (1,a3); 0 when flat or beyond +-1.5."""
    a1, a2, a3 = f32(a1), f32(a2), f32(a3)
    slope = f32(0.5 * float(f32(a3 - a1)))
    curve = f32(f32(a3 + a1) - f32(2) * a2)
    if curve == 0:
        return f32(0)
    peak = f32(-slope / curve)
    if peak > 1.5 or peak < -1.5:
        return f32(0)
    return peak


def determine_center(stacks: list[np.ndarray]) -> tuple[float, float, float]:
    """radialft.cpp:507-614 (non-I2M): the peak of the float32 phase average
    (first maximum in z, y, x order, only values > 0) refined by parabolas
    along z (nz > 1), y and x with wrap-around neighbours.  The reference's
    stack is nxExtra wide; its padding columns are zero, which only matters
    through the x wrap of a peak on column 0 (handled as the reference)."""
    nz, ny, nx = stacks[0].shape
    nxe = nx + 1 if nx % 2 else nx + 2
    avg = np.zeros((nz, ny, nxe), np.float32)
    for s in stacks:
        avg[:, :, :nx] += s
    avg /= f32(len(stacks))
    flat = int(np.argmax(avg))
    if avg.flat[flat] > 0:
        maxk, maxi, maxj = np.unravel_index(flat, avg.shape)
    else:
        maxk = maxi = maxj = 0
    maxval = avg[maxk, maxi, maxj] if avg.flat[flat] > 0 else f32(0)
    if nz > 1:
        zc = f32(maxk + fitparabola(avg[(maxk - 1) % nz, maxi, maxj], maxval, avg[(maxk + 1) % nz, maxi, maxj]))
    else:
        zc = f32(maxk)
    yc = f32(maxi + fitparabola(avg[maxk, (maxi - 1) % ny, maxj], maxval, avg[maxk, (maxi + 1) % ny, maxj]))
    xc = f32(maxj + fitparabola(avg[maxk, maxi, (maxj - 1) % nxe], maxval, avg[maxk, maxi, (maxj + 1) % nxe]))
    return float(xc), float(yc), float(zc)


def sep_matrix(nphases: int) -> np.ndarray:
    """radialft.cpp:440-452: M[band][phase] (float32), normalised by nphases."""
    norders = (nphases + 1) // 2
    phi = 2 * math.pi / nphases
    m = np.zeros((nphases, nphases), np.float32)
    for j in range(nphases):
        m[0, j] = f32(1.0 / nphases)
        for o in range(1, norders):
            m[2 * o - 1, j] = f32(math.cos(j * o * phi) / nphases)
            m[2 * o, j] = f32(math.sin(j * o * phi) / nphases)
    return m


def _signed(n: int) -> np.ndarray:
    k = np.arange(n)
    return np.where(k > n // 2, k - n, k)


def shift_center(band: np.ndarray, nx: int, xc: float, yc: float, zc: float) -> np.ndarray:
    """radialft.cpp:846-874: multiply the half spectrum [nz][ny][nx/2+1] by
    exp(i (dphiz kz + dphiy ky + dphix kx)) with float32 phases (moves the
    bead at (xc, yc, zc) to the origin)."""
    nz, ny, nxh = band.shape
    dphiz = f32(2 * math.pi * float(f32(zc)) / nz)
    dphiy = f32(2 * math.pi * float(f32(yc)) / ny)
    dphix = f32(2 * math.pi * float(f32(xc)) / nx)
    phi1 = (dphiz * _signed(nz).astype(np.float32))[:, None, None]
    phi2 = (dphiy * _signed(ny).astype(np.float32))[None, :, None]
    phi3 = (dphix * np.arange(nxh).astype(np.float32))[None, None, :]
    phi = ((phi1 + phi2).astype(np.float32) + phi3).astype(np.float32)
    rot = np.cos(phi).astype(np.float32) + 1j * np.sin(phi).astype(np.float32)
    return band * rot


def sphere_ft(k: np.ndarray, radius: float) -> np.ndarray:
    """radialft.cpp:1155-1167 (double): FT of a uniform sphere of the given
    radius at spatial frequency k."""
    k = np.asarray(k, np.float64)
    out = np.full(k.shape, 4 * math.pi * radius ** 3 / 3)
    nzm = k != 0
    x = 2 * math.pi * radius * k[nzm]
    out[nzm] = radius / (math.pi * k[nzm] * k[nzm]) * (np.sin(x) / x - np.cos(x))
    return out


def beadsize_ratio(order: int, norders: int, nx: int, ny: int, nz: int, dr: float, dz: float, angle: float,
                   ls: float, beaddiam: float) -> np.ndarray:
    """radialft.cpp:784-841: the float32 divisor of every element of the
    band(s) of one order: sphereFT(|k + k0_order|)/sphereFT(0), 1 at the
    origin of order 0."""
    dkx = f32(1.0 / float(f32(nx * f32(dr))))
    dky = f32(1.0 / float(f32(ny * f32(dr))))
    dkz = f32(1.0 / float(f32(nz * f32(dz))))
    k0mag = f32(f32(1) / f32(ls))
    radius = f32(float(f32(beaddiam)) * 0.5)
    limit = f32(4 * math.pi * float(radius) * float(radius) * float(radius) / 3)
    with np.errstate(divide="ignore", invalid="ignore"):
        ofrac = f32(f32(order) / f32(norders - 1)) if norders > 1 else f32(np.nan if order == 0 else np.inf)
    k0x = f32(f32(ofrac * k0mag) * f32(math.cos(float(f32(angle)))))
    k0y = f32(f32(ofrac * k0mag) * f32(math.sin(float(f32(angle)))))
    kz = (_signed(nz).astype(np.float32) * dkz)[:, None, None]
    ky = (_signed(ny).astype(np.float32) * dky + k0y).astype(np.float32)[None, :, None]
    kx = (np.arange(nx // 2 + 1).astype(np.float32) * dkx + k0x).astype(np.float32)[None, None, :]
    rho = np.sqrt(((kz * kz + ky * ky).astype(np.float32) + kx * kx).astype(np.float32)).astype(np.float32)
    ratio = (sphere_ft(rho, float(radius)) / float(limit)).astype(np.float32)
    if order == 0:
        ratio[0, 0, 0] = 1
    return ratio


def radial_average(band: np.ndarray, nx: int, ny: int, nz: int, dr: float, nr: int) -> np.ndarray:
    """radialft.cpp:876-936: bin the half spectrum by rint(|kxy|/dkr), mean per
    (bin, kz), then real at kz = 0 and Hermitian along kz.  Returns complex
    [nr/2+1][nz]."""
    nxh = nx // 2 + 1
    dkx = f32(f32(1) / f32(nx * f32(dr)))
    dky = f32(f32(1) / f32(ny * f32(dr)))
    maxk = f32(f32(0.5) / f32(dr))
    dkr = f32(f32(1) / f32(nr * f32(dr)))
    kyf = (_signed(ny).astype(np.float32) * dky)[:, None]
    kxf = (np.arange(nxh).astype(np.float32) * dkx)[None, :]
    rdist = np.sqrt((kxf * kxf + kyf * kyf).astype(np.float32)).astype(np.float32)
    inside = rdist < maxk
    indr = np.rint((rdist / dkr).astype(np.float32)).astype(np.int64)
    nbins = nr // 2 + 1
    idx = indr[inside]
    cnt = np.bincount(idx, minlength=nbins)[:nbins]
    # float32 sums in the reference's order (ky rows, then kx; np.add.at is
    # unbuffered and applies the indices in order)
    re = np.zeros((nbins, nz), np.float32)
    im = np.zeros((nbins, nz), np.float32)
    for kz in range(nz):
        vals = band[kz][inside].astype(np.complex64)
        np.add.at(re[:, kz], idx, vals.real)
        np.add.at(im[:, kz], idx, vals.imag)
    nzc = cnt > 0
    re[nzc] /= cnt[nzc, None].astype(np.float32)
    im[nzc] /= cnt[nzc, None].astype(np.float32)
    out = (re + 1j * im).astype(np.complex64)
    out[:, 0] = out[:, 0].real
    for kz in range(1, nz // 2 + 1):
        v = ((out[:, kz] + np.conj(out[:, nz - kz])) / np.float32(2)).astype(np.complex64)
        out[:, kz] = v
        out[:, nz - kz] = np.conj(v)
    return out


def modify(otf: np.ndarray, order: int, ifixz: int, ifixr: int) -> None:
    """radialft.cpp:1169-1186 on one [nkr][nz] band."""
    nz = otf.shape[1]
    if ifixz:
        for kz in range(nz):
            if kz != 0 or order > 0:
                otf[0, kz] = otf[1, kz]
    if ifixr:
        for kx in range(ifixr, otf.shape[0]):
            otf[kx, 0] = (otf[kx, 1] + otf[kx, nz - 1]) / 2


def cleanup(otf: np.ndarray, order: int, nr: int, nz: int, o: MakeOTFOptions) -> None:
    """radialft.cpp:938-999 (single objective): clear what lies outside the
    band's support along kz, keeping the leavekz pixels next to it."""
    lamda = f32(o.wavelength * 0.001)
    na, nimm = f32(o.na), f32(o.nimm)
    sinalpha = f32(na / nimm)
    cosalpha = f32(math.cos(math.asin(float(sinalpha))))
    krmax = f32(f32(2) * na / lamda)
    dkr = f32(1.0 / float(f32(nr * f32(o.dr))))
    dkz = f32(1.0 / float(f32(nz * f32(o.dz))))
    icleanup = otf.shape[0]
    for ix in range(icleanup):
        kr = f32(ix * dkr)
        if kr <= krmax:
            beta = f32(math.asin(float(f32(f32(na - f32(kr * lamda)) / nimm))))
            kzedge = f32(f32(nimm / lamda) * f32(f32(math.cos(float(beta))) - cosalpha))
            if order == 0:
                kzstart = int(np.rint(f32(f32(kzedge / dkz) + f32(1))))
                kzend = nz - kzstart
                for iz in range(kzstart, kzend + 1):
                    otf[ix, iz] = 0
            elif order == 1:
                jotf = int(np.rint(float(f32(kzedge / dkz)) + 0.999))
                kzend = o.leavekz[0] - jotf
                if kzend >= 0:
                    for iz in range(0, kzend + 1):
                        otf[ix, iz] = 0
                        if iz != 0:
                            otf[ix, nz - iz] = 0
                for iz in range(o.leavekz[1] + jotf + 1, nz // 2 + 1):
                    otf[ix, iz] = 0
                    otf[ix, nz - iz] = 0
            else:
                jotf = int(np.rint(float(f32(kzedge / dkz)) + 0.999))
                for iz in range(o.leavekz[2] + jotf, nz // 2 + 1):
                    otf[ix, iz] = 0
                    otf[ix, nz - iz] = 0
        else:
            otf[ix, :] = 0


def fixorigin(otf: np.ndarray, kx1: int, kx2: int) -> None:
    """radialft.cpp:1188-1224 on band 0: replace the kz = 0 values of kr < kx1
    with a straight-line fit (in kr) of the kz-summed real parts over
    [kx1, kx2]."""
    meani = f32(0.5 * (kx1 + kx2))
    numvals = kx2 - kx1 + 1
    sums = np.zeros(kx2 + 1)
    totsum = ysum = sqsum = 0.0
    for i in range(kx2 + 1):
        sums[i] = float(otf[0, 0].real) if i == 0 else float(np.sum(otf[i, :].real.astype(np.float64)))
        if i >= kx1:
            d = f32(f32(i) - meani)
            totsum += sums[i]
            ysum += sums[i] * float(d)
            sqsum += float(f32(d * d))
    slope = f32(ysum / sqsum)
    avg = f32(totsum / numvals)
    for i in range(kx1):
        lineval = f32(avg + f32(f32(f32(i) - meani) * slope))
        otf[i, 0] = complex(float(f32(float(f32(otf[i, 0].real)) - (sums[i] - float(lineval)))), otf[i, 0].imag)


def combine_reim(bands: list[np.ndarray], norders: int, nx: int, nz: int, pishift: bool) -> None:
    """radialft.cpp:746-782: rotate each side band pair (re, im) by the phase
    phi estimated from their magnitude sums and the kz = 0 signs at kr = nx/4,
    keep band re' = re cos(phi) - im sin(phi), clear band im."""
    for o in range(1, norders):
        re_b, im_b = bands[2 * o - 1], bands[2 * o]
        re_mag = float(np.sum(np.abs(re_b.astype(np.complex64)).astype(np.float64)))
        im_mag = float(np.sum(np.abs(im_b.astype(np.complex64)).astype(np.float64)))
        phi = math.atan(im_mag / re_mag)
        r0, i0 = re_b[nx // 4, 0].real, im_b[nx // 4, 0].real
        if r0 < 0 and i0 > 0:
            phi += math.pi
        elif r0 < 0 and i0 < 0:
            phi = math.pi - phi
        elif r0 > 0 and i0 > 0:
            phi = -phi
        if o == 1 and pishift:
            phi = math.pi - phi
        bands[2 * o - 1] = re_b * float(f32(math.cos(phi))) + im_b * float(f32(math.sin(-phi)))
        bands[2 * o] = np.zeros_like(im_b)


def makeotf(psf: np.ndarray, opts: MakeOTFOptions) -> np.ndarray:
    """radialft.cpp main (154-418) on an in-memory PSF stack float32
    [nz*nphases][ny][nx] (phase fastest).  Returns the OTF file contents,
    float32 [nbands_out][nx/2+1][2*nz] (complex kz along a row)."""
    psf = np.array(psf, dtype=np.float32, copy=True)
    nsec, ny, nx = psf.shape
    nph = opts.nphases
    if nx > ny:
        raise ValueError("PSF width larger than its height is not supported (the reference overruns its buffers)")
    nz = nsec // nph
    norders = (nph + 1) // 2
    bg = np.zeros(nz * nph, np.float32)
    floatimage = [np.zeros((nz, ny, nx), np.float32) for _ in range(nph)]
    for z in range(nz):
        for p in range(nph):
            zsec = z * nph + p
            sec = psf[zsec]
            if sec[ny - 1, nx - 1] < 0:  # camera fix (228-230)
                sec[ny - 1, nx - 1] = sec[ny - 1, nx - 2]
            bg[zsec] = f32(opts.background) if opts.background >= 0 else estimate_background(sec)
            img = sec.copy()
            apodize(img)
            floatimage[p][z] = img
    xc, yc, zc = determine_center(floatimage)
    for z in range(nz):
        for p in range(nph):
            floatimage[p][z] -= bg[z * nph + p]
    if nph > 1:
        m = sep_matrix(nph)
        out = []
        for i in range(nph):
            acc = np.zeros((nz, ny, nx), np.float32)
            for j in range(nph):
                acc += floatimage[j] * m[i, j]
            out.append(acc)
        floatimage = out
    bands = [np.fft.rfftn(f.astype(np.float64)).astype(np.complex64) for f in floatimage]
    bands = [shift_center(b, nx, xc, yc, zc) for b in bands]
    if opts.compensate:
        for o in range(norders):
            r = beadsize_ratio(o, norders, nx, ny, nz, opts.dr, opts.dz, opts.angle, opts.ls, opts.beaddiam)
            if o == 0:
                bands[0] = bands[0] / r
            else:
                bands[2 * o - 1] = bands[2 * o - 1] / r
                bands[2 * o] = bands[2 * o] / r
    nr = min(nx, ny)
    avg = [radial_average(b, nx, ny, nz, opts.dr, nr) for b in bands]
    scalefactor = 1.0
    for p in range(nph):
        order = (p + 1) // 2
        modify(avg[p], order, opts.ifixz, opts.ifixr)
        if opts.bessel:
            pass
        elif opts.leavekz[0] > 0:
            cleanup(avg[p], order, nr, nz, opts)
        if p == 0 and opts.fixorigin[0] > 0:
            fixorigin(avg[p], opts.fixorigin[0], opts.fixorigin[1])
        if order == 0 or opts.rescale:
            scalefactor = float(f32(f32(1) / f32(avg[p][0, 0].real)))
        avg[p] = avg[p] * scalefactor
    if not opts.five_bands and nph > 1:
        combine_reim(avg, norders, nx, nz, opts.pishift)
    if opts.conj:
        avg = [np.conj(a) for a in avg]
    sel = list(range(nph)) if opts.five_bands else [0] + [2 * o - 1 for o in range(1, norders)]
    nxh = nx // 2 + 1
    out = np.zeros((len(sel), nxh, 2 * nz), np.float32)
    for i, b in enumerate(sel):
        out[i, :, 0::2] = avg[b].real
        out[i, :, 1::2] = avg[b].imag
    if nz == 1:
        out = out.reshape(len(sel), 1, 2 * nxh)
    return out
