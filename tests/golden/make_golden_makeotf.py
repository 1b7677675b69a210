"""Generates the makeotf golden fixtures tests/golden/mo_<case>.npz.

Each fixture holds a synthetic bead PSF stack (uint16, phase-fastest
sections), the makeotf switches, and the OTF array the reference program
writes for them: src/otf/radialft.cpp compiled unmodified and run
in-process by oracle/makeotf_ref.py (FFTW's float r2c replaced by a
double-precision DFT, see oracle/ref_harness/makeotf_harness.cpp).  Run
from the repository root where the reference checkout is available:

    python tests/golden/make_golden_makeotf.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from cudasirecon_gb300.synthetic import Optics, bead_psf_stack  # noqa: E402

BASE = ["-angle", "-0.8043", "-ls", "0.2035", "-xyres", "0.08", "-zres", "0.125", "-na", "1.42", "-nimm", "1.515",
        "-wavelength", "528"]


def cases():
    o = Optics()
    psf64 = bead_psf_stack(64, 64, 32, o, peak_photons=3e4, seed=11)
    psf48 = bead_psf_stack(48, 64, 24, o, peak_photons=3e4, seed=12, offset_px=(-0.4, 0.35, -0.3),
                           pattern_phase=2.0)
    psf2d = bead_psf_stack(64, 64, 1, Optics(nphases=3), nphases=3, peak_photons=3e4, seed=13)
    return {
        "mo3d_64": (psf64, BASE + ["-fixorigin", "3", "20"]),
        "mo3d_64_clean": (psf64, BASE + ["-leavekz", "7", "11", "3", "-nocompen", "-5bands"]),
        # bead 0.1 um: the first zero of its transform (radialft.cpp:1155-1167)
        # stays outside the sampled |k + k0| (a 0.2 um bead divides by ~0 there)
        "mo3d_64_misc": (psf64, BASE + ["-background", "100", "-rescale", "-conj", "-ifixkr", "5", "-beaddiam",
                                        "0.1"]),
        "mo3d_48x64": (psf48, BASE + ["-fixorigin", "3", "12", "-PIshift"]),
        "mo2d_64": (psf2d, BASE + ["-nphases", "3", "-fixorigin", "3", "20"]),
    }


def main() -> None:
    import build_ref  # noqa: F401
    import makeotf_ref

    if not build_ref.build_makeotf():
        raise SystemExit("reference makeotf could not be built")
    out_dir = os.path.dirname(os.path.abspath(__file__))
    for name, (psf, args) in cases().items():
        psf16 = np.clip(np.rint(psf), 0, 65535).astype(np.uint16)
        otf = makeotf_ref.run(psf16.astype(np.float32), args)
        np.savez_compressed(os.path.join(out_dir, f"mo_{name}.npz"), psf=psf16, args=np.array(args), otf=otf)
        print(name, psf16.shape, otf.shape)


if __name__ == "__main__":
    main()
