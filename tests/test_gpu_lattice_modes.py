"""GPU parity of the load-stage and light-sheet modes against the
reference's own CUDA build (oracle/refharness, whose host loading restates
setup_common and loadImageData): cropXY (cudaSirecon.cpp:1165-1168), deskew
with a shift (1153-1161, deskewOneSection 1733-1760), Bessel-sheet SIM
(gpuFunctionsImpl.cu:317-323, 503-556, 883-885, 1260-1294, 1569-1577) with and
without noRecon (cudaSirecon.cpp:1325), and the per-section extra background
of the DV extended header (bBgInExtHdr, 1386-1393) through the CLI.  Bar: the
parity tolerances (volume rel-L2 <= 1e-4, max-abs <= 1e-3 of the peak, k0
within 1e-3 px, modamps within 1e-3)."""
import os
import struct
import subprocess

import numpy as np
import pytest

import cudasirecon_gb300 as sr

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def refmod():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("the reference CUDA build could not be compiled")
    from oracle import refharness
    return refharness


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


@pytest.fixture(scope="module")
def data3d():
    from cudasirecon_gb300 import synthetic as syn
    o = syn.Optics()
    raw = syn.simulate(128, 128, 16, o, seed=17, n_filaments=20).raw
    return raw, syn.ra_otf(o, nx_psf=128, nz_psf=64), syn.config_text(o)


def both(refmod, raw, otf, cfg, nx, bg=None):
    r = sr.Reconstructor(nx, nx, raw.shape[0], cfg, otf)
    r.set_raw(raw)
    r.load_and_rescale(0, 0)
    r.set_cur_time(0)
    r.process()
    got, (k0, amp) = r.result().copy(), r.fit()
    ref = refmod.RefRecon(nx, nx, raw.shape[0], cfg, otf)
    if bg is not None:
        ref.set_section_backgrounds(bg)
    ref.set_raw(raw.astype(np.float32))
    ref.load_and_rescale(0)
    ref.set_cur_time(0)
    ref.process()
    want, (rk0, ramp) = ref.result().copy(), ref.fit()
    shape = (r.out_shape, ref.out_shape, r.nx_recon)
    r.close()
    ref.close()
    return got, want, k0, rk0, amp, ramp, shape


def check(got, want, k0, rk0, amp, ramp, nxr, dxy=0.08):
    assert got.shape == want.shape
    assert np.isfinite(got).all()
    rel = rel_l2(got, want)
    assert rel <= 1e-4, rel
    assert np.abs(got - want).max() <= 1e-3 * np.abs(want).max()
    assert np.abs(k0 - rk0).max() * nxr * dxy <= 1e-3
    assert np.abs(amp - ramp).max() <= 1e-3


def test_cropxy_matches_reference(refmod, data3d):
    raw, otf, cfg = data3d
    got, want, k0, rk0, amp, ramp, (s1, s2, nxr) = both(refmod, raw, otf, cfg + "\ncropXY=96\n", 128)
    assert nxr == 96 and s1 == s2 == (16, 256, 192)
    check(got, want, k0, rk0, amp, ramp, nxr)


def test_deskew_with_shift_matches_reference(refmod, data3d):
    raw, otf, cfg = data3d
    # 128 + 16 cos(28.3 deg) 0.125 / 0.08 = 150.0 -> 150 = 2 3 5^2 columns after deskewing
    got, want, k0, rk0, amp, ramp, (s1, s2, nxr) = both(refmod, raw, otf, cfg + "\ndeskew=28.3\ndeskewshift=3\n", 128)
    assert nxr == 150 and s1 == s2
    check(got, want, k0, rk0, amp, ramp, nxr)


@pytest.mark.parametrize("norecon", [False, True])
def test_bessel_mode_matches_reference(refmod, data3d, norecon):
    raw, otf, cfg = data3d
    # the pattern must lie inside the Bessel beam's axial extent, k0 <= 2 NA / lambda_ex
    # (2.46 <= 2.66 1/um here); beyond it the reference's half angle is acos(> 1) = NaN and
    # its plane count (int)NaN is undefined
    extra = "\nbessel=1\nbesselNA=0.65\nbesselExWave=0.488\n" + ("noRecon=1\n" if norecon else "")
    got, want, k0, rk0, amp, ramp, (_, _, nxr) = both(refmod, raw, otf, cfg + extra, 128)
    check(got, want, k0, rk0, amp, ramp, nxr)


def write_dv_ext(path, stack, dxy, dz, wave, section_bg):
    """DV file whose extended header holds, per section, 2 ints and 3 floats
    with the section's extra background as the third float."""
    nz, ny, nx = stack.shape
    nint, nreal = 2, 3
    ext = bytearray()
    for s in range(nz):
        ext += struct.pack("<2i", s, 7) + struct.pack("<3f", 1.5, -2.0, float(section_bg[s]))
    h = bytearray(1024)
    struct.pack_into("<4i", h, 0, nx, ny, nz, 2)
    struct.pack_into("<3f", h, 40, dxy, dxy, dz)
    struct.pack_into("<3i", h, 64, 1, 2, 3)
    struct.pack_into("<i", h, 92, len(ext))
    struct.pack_into("<h", h, 96, -16224)
    struct.pack_into("<hh", h, 128, nint, nreal)
    struct.pack_into("<hh", h, 196, 1, wave)
    with open(path, "wb") as f:
        f.write(bytes(h) + bytes(ext))
        f.write(np.ascontiguousarray(stack, np.float32).tobytes())


def test_background_from_extended_header_matches_reference(refmod, tmp_path):
    from golden_cases import load
    case, _ = load("c3d_64")
    raw = case["raw"][0].astype(np.float32)
    bg = np.random.default_rng(5).uniform(0.0, 20.0, raw.shape[0]).astype(np.float32)
    inp, out = tmp_path / "cell.dv", tmp_path / "cell_proc.dv"
    write_dv_ext(inp, raw, 0.08, 0.125, 528, bg)
    otf = tmp_path / "otf.tif"
    sr.load_library()
    sr.write_tiff_float(str(otf), case["otf"])
    cfg = tmp_path / "config"
    cfg.write_text(case["config"] + "\nbgInExtHdr=1\n")
    exe = os.path.join(ROOT, "cudasirecon_gb300", "bin", "cudasirecon")
    r = subprocess.run([exe, str(inp), str(out), str(otf), "-c", str(cfg)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0 and "Error" not in r.stderr, r.stderr
    with open(out, "rb") as f:
        h = f.read(1024)
        nx, ny, nz = struct.unpack_from("<3i", h, 0)
        got = np.frombuffer(f.read(), np.float32).reshape(nz, ny, nx)
    ref = refmod.RefRecon(case["nx"], case["ny"], raw.shape[0], case["config"] + "\nbgInExtHdr=1\n", case["otf"])
    ref.set_section_backgrounds(bg)
    ref.set_raw(raw)
    ref.load_and_rescale(0)
    ref.set_cur_time(0)
    ref.process()
    want = ref.result()
    ref.close()
    # the backgrounds change the result (so they were read) ...
    plain = refmod.RefRecon(case["nx"], case["ny"], raw.shape[0], case["config"], case["otf"])
    plain.set_raw(raw)
    plain.load_and_rescale(0)
    plain.set_cur_time(0)
    plain.process()
    assert rel_l2(plain.result(), want) > 1e-3
    plain.close()
    # ... and the product subtracts the same ones
    assert rel_l2(got, want) <= 1e-4
