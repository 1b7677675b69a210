"""makeotf oracle (oracle/makeotf_oracle.py) against the reference program's
own outputs (tests/golden/mo_*.npz, made by running src/otf/radialft.cpp
compiled unmodified; see tests/golden/make_golden_makeotf.py), plus the
OTF properties makeotf guarantees.  CPU only."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import makeotf_oracle as mo  # noqa: E402

FIXTURES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "mo_*.npz")))
# oracle vs reference: float64 FFT and bin sums against the reference's float32
REL_L2 = 1e-5
MAX_ABS = 1e-5


def load(path):
    z = np.load(path)
    return z["psf"].astype(np.float32), [str(a) for a in z["args"]], z["otf"]


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[3:-4] for p in FIXTURES])
def test_oracle_matches_reference_program(path):
    psf, args, ref = load(path)
    got = mo.makeotf(psf, mo.MakeOTFOptions.from_args(args))
    assert got.shape == ref.shape
    d = got - ref
    assert np.linalg.norm(d) / np.linalg.norm(ref) <= REL_L2
    assert np.abs(d).max() <= MAX_ABS


def test_fixture_set_complete():
    names = {os.path.basename(p)[3:-4] for p in FIXTURES}
    assert {"mo3d_64", "mo3d_64_clean", "mo3d_64_misc", "mo3d_48x64", "mo2d_64"} <= names


def test_otf_properties():
    """Band 0 is 1 at the origin (rescale), real on the kz = 0 plane, and
    every band is Hermitian along kz (radialft.cpp:923-934)."""
    psf, args, ref = load(os.path.join(ROOT, "tests", "golden", "mo_mo3d_64.npz"))
    c = ref[..., 0::2] + 1j * ref[..., 1::2]
    nz = c.shape[2]
    assert abs(c[0, 0, 0] - 1) < 1e-6
    assert np.abs(c[:, :, 0].imag).max() == 0
    kz = np.arange(1, nz)
    assert np.allclose(c[:, :, kz], np.conj(c[:, :, nz - kz]), atol=1e-7)


def test_options_parse_defaults_and_switches():
    o = mo.MakeOTFOptions.from_args([])
    assert (o.nphases, o.angle, o.ls, o.dr, o.dz, o.wavelength) == (5, 1.57, 0.2, 0.106, 0.1, 525)
    o = mo.MakeOTFOptions.from_args(["-fixorigin", "3", "20", "-leavekz", "1", "2", "3", "-nocompen", "-5bands"])
    assert o.fixorigin == (3, 20) and o.leavekz == (1, 2, 3) and not o.compensate and o.five_bands
    with pytest.raises(ValueError):
        mo.MakeOTFOptions.from_args(["-2lenses"])


def test_separation_matrix_inverts_phase_stepping():
    """sep_matrix (radialft.cpp:440-452) applied to a pure order-o stepping
    returns that order's cos/sin parts."""
    m = mo.sep_matrix(5).astype(np.float64)
    ph = 2 * np.pi * np.arange(5) / 5
    for o in (1, 2):
        a = m @ np.cos(o * ph + 0.3)
        assert abs(a[2 * o - 1] - 0.5 * np.cos(0.3)) < 1e-6
        assert abs(a[2 * o] + 0.5 * np.sin(0.3)) < 1e-6
    assert abs((m @ np.ones(5))[0] - 1) < 1e-6


def test_center_finds_subpixel_bead():
    from cudasirecon_gb300.synthetic import bead_psf_stack
    psf = bead_psf_stack(64, 64, 32, peak_photons=1e6, seed=3, offset_px=(0.25, -0.3, 0.2))
    stacks = [psf[p::5].copy() for p in range(5)]
    for s in stacks:
        for z in range(s.shape[0]):
            mo.apodize(s[z])
    xc, yc, zc = mo.determine_center(stacks)
    assert abs(xc - 32.25) < 0.15 and abs(yc - 31.7) < 0.15 and abs(zc - 16.2) < 0.15
