"""GPU parity at the sizes where the fast kernel paths run (256- to 1024-point
lines, nz a multiple of 16): the product against the reference's own CUDA
build (oracle/refharness: gpuFunctionsImpl.cu compiled unmodified) on seeded
synthetic acquisitions, both run live on the GPU.

Each case runs two time points: t = 0 searches k0, t = 1 reuses it (the
time-series path the benchmark measures); the second also goes through
SRX_processSeries.  Tolerances are the parity bar: volume rel-L2 <= 1e-4,
max-abs <= 1e-3 of the peak, k0 within 1e-3 px, modamps within 1e-3.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make(nx, ny, nz, nt, seed):
    from cudasirecon_gb300 import synthetic as syn
    o = syn.Optics()
    vols = [syn.simulate(nx, ny, nz, o, seed=seed, drift_px=0.2 * t, bleach=0.99 ** t, noise_seed=1000 + t,
                         scene_seed=seed, mod_seed=seed + 1, n_filaments=30).raw for t in range(nt)]
    return vols, syn.ra_otf(o, nx_psf=128, nz_psf=64), syn.config_text(o)


@pytest.fixture(scope="module")
def refmod():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("the reference CUDA build could not be compiled")
    from oracle import refharness
    return refharness


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def run_both(refmod, nx, ny, nz, nt=2, seed=5):
    import cudasirecon_gb300 as sr
    vols, otf, cfg = make(nx, ny, nz, nt, seed)
    nimg = vols[0].shape[0]
    ref = refmod.RefRecon(nx, ny, nimg, cfg, otf)
    ref.set_ntimes(nt)
    r = sr.Reconstructor(nx, ny, nimg, cfg, otf)
    r.set_ntimes(nt)
    want, got, fits = [], [], []
    for t in range(nt):
        ref.set_raw(vols[t].astype(np.float32))
        ref.load_and_rescale(t)
        ref.set_cur_time(t)
        ref.process()
        want.append(ref.result().copy())
        r.set_raw(vols[t])
        r.load_and_rescale(t, 0)
        r.set_cur_time(t)
        r.process()
        got.append(r.result().copy())
        fits.append((r.fit(), ref.fit()))
    ref.close()
    return vols, r, want, got, fits


def check(nx, got, want, fits, dxy=0.08):
    dk = 1.0 / (nx * dxy)
    for t, (g, w) in enumerate(zip(got, want)):
        assert np.isfinite(g).all()
        assert rel_l2(g, w) < 1e-4, f"t={t}: rel-L2 {rel_l2(g, w):.3g}"
        assert np.abs(g - w).max() / np.abs(w).max() < 1e-3
    for (k0, amp), (rk0, ramp) in fits:
        assert np.abs(np.asarray(k0) - np.asarray(rk0)).max() / dk < 1e-3
        assert np.abs(np.asarray(amp) - np.asarray(ramp)).max() < 1e-3


@pytest.mark.parametrize("shape", [(256, 256, 32), (512, 512, 48)], ids=["256x256x32", "512x512x48"])
def test_fast_paths_match_reference_kernels(refmod, shape):
    nx, ny, nz = shape
    vols, r, want, got, fits = run_both(refmod, nx, ny, nz)
    check(nx, got, want, fits)
    # the time-series entry point gives the same volumes
    outs = [np.zeros(r.out_shape, np.float32) for _ in vols]
    r.process_series([np.ascontiguousarray(v) for v in vols], outs, t0=0)
    for t in range(len(vols)):
        assert np.array_equal(outs[t], got[t])
    r.close()


def test_separated_bands_match_reference_kernels(refmod):
    """Ingest (flat-field, apodisation, x/y FFT), bleach correction and the
    separation + z FFT at 256^2 x 32, band by band."""
    import cudasirecon_gb300 as sr
    vols, otf, cfg = make(256, 256, 32, 1, 7)
    nimg = vols[0].shape[0]
    ref = refmod.RefRecon(256, 256, nimg, cfg, otf)
    ref.set_raw(vols[0].astype(np.float32))
    ref.load_and_rescale(0)
    ref.stage_separate()
    r = sr.Reconstructor(256, 256, nimg, cfg, otf)
    r.set_raw(vols[0])
    r.load_and_rescale(0, 0)
    r.prepare()
    for d in range(3):
        for b in range(5):
            assert rel_l2(r.band(d, b), ref.band(d, b)) < 2e-5, (d, b)
    ref.close()
    r.close()
