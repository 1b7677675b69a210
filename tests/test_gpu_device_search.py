"""GPU: the k0 search on the device (k_findk0_finish + the cluster search
k_k0_search, the default) against the host-driven search (batched candidate
evaluations, one synchronisation per batch) on the same volumes.

Both visit the same float32 angle and magnitude sequences and make the same
float decisions and parabola fits; the candidate vectors come from the
device's cosf/sinf/atan2f on one side and the host libm on the other, and
the phase tables from float sincospi of an exactly reduced argument on one
side and double sincos on the other.  So the fitted k0 agree to about 1e-5
pixel, the amplitudes to float precision, and the volumes to a few 1e-6.
Parity of the device search with the reference itself is what every other
reconstruction test checks (it is the default path).
"""
import numpy as np
import pytest

import cudasirecon_gb300 as sr

pytestmark = pytest.mark.gpu


def case(nx, ny, nz, twod, seed):
    from cudasirecon_gb300 import synthetic as syn
    o = syn.Optics(nphases=3 if twod else 5)
    raw = syn.simulate(nx, ny, nz, o, seed=seed, n_filaments=10).raw
    otf = syn.ra_otf(o, nx_psf=128, nz_psf=64, norders=2 if twod else 3, twod=twod)
    cfg = syn.config_text(o, twod=twod, extra={"wiener": 0.00048828125} if twod else None)
    return raw, otf, cfg


def run(raw, otf, cfg, nx, ny, device):
    r = sr.Reconstructor(nx, ny, raw.shape[0], cfg, otf)
    r.set_device_search(device)
    r.set_raw(raw)
    r.load_and_rescale(0, 0)
    r.set_cur_time(0)
    c0 = r.fit_counts()
    r.process()
    c1 = r.fit_counts()
    out = r.result().copy()
    k0, amps = r.fit()
    r.close()
    return out, np.asarray(k0, np.float64), np.asarray(amps), {k: c1[k] - c0[k] for k in c1}


@pytest.mark.parametrize("nx,ny,nz,twod", [(128, 128, 16, False), (256, 256, 16, False), (256, 192, 24, False),
                                           (512, 512, 8, False), (128, 128, 1, True), (1024, 1024, 1, True)])
def test_device_search_matches_host_search(nx, ny, nz, twod):
    raw, otf, cfg = case(nx, ny, nz, twod, seed=7 + nx + nz)
    a, ka, ma, ca = run(raw, otf, cfg, nx, ny, True)
    b, kb, mb, cb = run(raw, otf, cfg, nx, ny, False)
    dk = 1.0 / (max(nx, ny) * 0.08)
    kdiff = float(np.abs(ka - kb).max() / dk)
    rel = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    adiff = float(np.abs(ma - mb).max())
    print(f"\n{nx}x{ny}x{nz}: k0 {kdiff:.2e} px, amps {adiff:.2e}, volume rel-L2 {rel:.2e}, "
          f"candidates device {ca['reductions']} host {cb['reductions']}")
    assert ca["k0_searches"] == cb["k0_searches"] == 3
    assert kdiff < 2e-4, kdiff
    assert adiff < 1e-4, adiff
    assert np.isfinite(a).all()
    assert rel < 5e-5, rel


def test_device_search_deterministic():
    raw, otf, cfg = case(256, 256, 16, False, seed=3)
    a, ka, ma, _ = run(raw, otf, cfg, 256, 256, True)
    b, kb, mb, _ = run(raw, otf, cfg, 256, 256, True)
    assert np.array_equal(ka, kb) and np.array_equal(ma, mb) and np.array_equal(a, b)
