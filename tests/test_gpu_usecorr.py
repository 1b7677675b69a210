"""Flat-field correction from a calibration file (the `usecorr` option,
bgAndSlope / getbg_and_slope, cudaSirecon.cpp:139-192): an MRC file of the
data's nx x ny whose first section is the per-pixel background and second the
per-pixel slope; ingest applies (raw - background) * slope."""
import struct

import numpy as np
import pytest

import cudasirecon_gb300 as sr
from golden_cases import load, rel_l2

pytestmark = pytest.mark.gpu


def write_mrc(path, stack):
    """float32 [nz][ny][nx] as MRC (mode 2, DV byte-order stamp, no extended header)"""
    nz, ny, nx = stack.shape
    h = bytearray(1024)
    struct.pack_into("<4i", h, 0, nx, ny, nz, 2)
    struct.pack_into("<h", h, 96, -16224)
    with open(path, "wb") as f:
        f.write(bytes(h))
        f.write(np.ascontiguousarray(stack, np.float32).tobytes())


def recon(case, cfg, raw):
    r = sr.Reconstructor(case["nx"], case["ny"], raw.shape[0], cfg, case["otf"])
    r.set_raw(raw)
    r.load_and_rescale(0, 0)
    r.set_cur_time(0)
    r.process()
    out = r.result().copy()
    r.close()
    return out


def test_calibration_file_equals_host_side_correction(tmp_path):
    case, _ = load("c3d_64")
    raw = case["raw"][0].astype(np.float32)
    ny, nx = raw.shape[1:]
    rng = np.random.default_rng(3)
    bg = (100 + 5 * rng.standard_normal((ny, nx))).astype(np.float32)
    slope = (1 + 0.05 * rng.standard_normal((ny, nx))).astype(np.float32)
    path = tmp_path / "corr.mrc"
    write_mrc(path, np.stack([bg, slope]))
    got = recon(case, case["config"] + f"\nusecorr={path}\n", raw)
    # the same correction applied on the host (float32, same operation order),
    # with no constant background
    pre = ((raw - bg[None]) * slope[None]).astype(np.float32)
    cfg0 = "\n".join(l for l in case["config"].splitlines() if not l.startswith("background=")) + "\nbackground=0\n"
    want = recon(case, cfg0, pre)
    assert np.isfinite(got).all()
    assert rel_l2(got, want) < 1e-6
    # and it differs from ignoring the calibration
    assert rel_l2(recon(case, case["config"], raw), want) > 1e-3


def test_calibration_file_of_another_size_is_refused(tmp_path):
    case, _ = load("c3d_64")
    path = tmp_path / "corr.mrc"
    write_mrc(path, np.ones((2, 32, 32), np.float32))
    with pytest.raises(sr.SIReconError, match="different dimension"):
        sr.Reconstructor(case["nx"], case["ny"], case["raw"].shape[1], case["config"] + f"\nusecorr={path}\n",
                         case["otf"])
