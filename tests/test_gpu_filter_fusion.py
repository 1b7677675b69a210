"""GPU: the Wiener filter applied inside the assembly's band load (default)
against the same filter run as its own in-place pass over the bands (the
reference's filterbands structure), on the same volume and the same fit.

The two paths evaluate the same filter scales at the same pixels; they differ
only in float rounding (the fused path multiplies the plus/conjugate part by
its scale directly instead of splitting the stored pair into plus and minus
and back), so the volumes agree to float precision.  Parity of the fused path
with the reference itself is covered at 256^2 x 32 and 512^2 x 48 by
test_gpu_parity_large.py and, in 2D, by the golden fixture c2d_128.
"""
import numpy as np
import pytest

import cudasirecon_gb300 as sr

pytestmark = pytest.mark.gpu


def case(nx, nz, twod, seed):
    from cudasirecon_gb300 import synthetic as syn
    o = syn.Optics(nphases=3 if twod else 5)
    raw = syn.simulate(nx, nx, nz, o, seed=seed, n_filaments=10).raw
    otf = syn.ra_otf(o, nx_psf=128, nz_psf=64, norders=2 if twod else 3, twod=twod)
    cfg = syn.config_text(o, twod=twod, extra={"wiener": 0.00048828125} if twod else None)
    return raw, otf, cfg


def run(raw, otf, cfg, nx, fused, extra=None):
    if extra:  # the case's switches replace the config's own lines
        keys = {ln.split("=")[0] for ln in extra.splitlines()}
        cfg = "\n".join(ln for ln in cfg.splitlines() if ln.split("=")[0] not in keys) + "\n" + extra
    r = sr.Reconstructor(nx, nx, raw.shape[0], cfg, otf)
    r.set_filter_fusion(fused)
    r.set_raw(raw)
    r.load_and_rescale(0, 0)
    r.set_cur_time(0)
    r.process()
    out = r.result().copy()
    fit = r.fit()
    r.close()
    return out, fit


@pytest.mark.parametrize("nx,nz,twod", [(128, 16, False), (256, 16, False), (128, 1, True), (256, 1, True)])
@pytest.mark.parametrize("extra", [None, "nofilterovlps=0\n", "dampenOrder0=0\n", "dampenOrder0=0\nnosuppress=0\n"],
                         ids=["default", "nofilterovlps", "nodampen", "nodampen-nosuppress"])
def test_fused_filter_matches_separate_pass(nx, nz, twod, extra):
    raw, otf, cfg = case(nx, nz, twod, seed=11 + nx + nz)
    a, fa = run(raw, otf, cfg, nx, True, extra)
    b, fb = run(raw, otf, cfg, nx, False, extra)
    assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[1], fb[1])  # the fit is untouched
    assert np.isfinite(a).all()
    rel = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    assert rel < 2e-6, rel
    assert float(np.abs(a - b).max()) <= 2e-5 * float(np.abs(b).max())
