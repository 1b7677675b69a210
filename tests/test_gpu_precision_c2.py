"""GPU precision at the large configuration: 1024 x 1024 px x 64 z x 15
images (uint16, the seeded synthetic generator of the time-series workload at
the large size), one standalone volume with its k0 search.

Full size: the product (CUDA, through the C ABI) against the reference's own
CUDA build (oracle/refharness: gpuFunctionsImpl.cu compiled unmodified), at
the parity bar -- volume rel-L2 <= 1e-4, max-abs <= 1e-3 of the peak, k0
within 1e-3 px, modamps within 1e-3.  A 256 x 256 lateral centre crop of the
same stack (all z planes) also runs the FP64 oracle (oracle/sirecon_oracle.py)
with the same bar.  The achieved figures are printed (pytest -s shows them).
Generating the stack takes about a minute.
"""
import json
import time
import warnings

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, DEPTH, DXY = 1024, 64, 0.08


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def compare(a, b, nx):
    (va, ka, ma), (vb, kb, mb) = a, b
    dk = 1.0 / (nx * DXY)
    return {"rel_l2": rel_l2(va, vb), "max_abs_of_peak": float(np.abs(va - vb).max() / np.abs(vb).max()),
            "k0_px": float(np.abs(np.asarray(ka, np.float64) - np.asarray(kb, np.float64)).max() / dk),
            "modamp": float(np.abs(np.asarray(ma) - np.asarray(mb)).max())}


def bar(c):
    return c["rel_l2"] <= 1e-4 and c["max_abs_of_peak"] <= 1e-3 and c["k0_px"] <= 1e-3 and c["modamp"] <= 1e-3


def product(raw, cfg, otf, nx):
    import cudasirecon_gb300 as sr
    r = sr.Reconstructor(nx, nx, raw.shape[0], cfg, otf)
    r.set_raw(raw)
    r.load_and_rescale(0, 0)
    r.set_cur_time(0)
    r.process()
    out = (r.result().copy(), *r.fit())
    r.close()
    return out


def reference(raw, cfg, otf, nx):
    from oracle import refharness
    ref = refharness.RefRecon(nx, nx, raw.shape[0], cfg, otf)
    ref.set_raw(raw.astype(np.float32))
    ref.load_and_rescale(0)
    ref.set_cur_time(0)
    ref.process()
    out = (ref.result().copy(), *ref.fit())
    ref.close()
    return out


def fp64(raw, cfg, otf, nx):
    from oracle.sirecon_oracle import SIMReconOracle
    o = SIMReconOracle(nx, nx, raw.shape[0], cfg, otf)
    o.set_raw(raw)
    o.load_and_rescale(0)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        o.process()
    return np.asarray(o.result, np.float64), np.asarray(o.k0), np.asarray(o.amp)


@pytest.fixture(scope="module")
def stack():
    from cudasirecon_gb300 import synthetic as syn
    o = syn.Optics()
    t = time.perf_counter()
    raw = syn.simulate(N, N, DEPTH, o, seed=2).raw
    return raw, syn.config_text(o), syn.ra_otf(o, nx_psf=128, nz_psf=64), time.perf_counter() - t


def test_precision_1024x1024x64_against_reference_build(stack):
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("the reference CUDA build could not be compiled")
    raw, cfg, otf, gen_s = stack
    c = compare(product(raw, cfg, otf, N), reference(raw, cfg, otf, N), N)
    print("\nC2 1024^2x64 product vs reference CUDA build:", json.dumps(c), f"(stack generated in {gen_s:.0f} s)")
    assert bar(c), c


def test_precision_crop_against_fp64_oracle(stack):
    from oracle import build_ref
    raw, cfg, otf, _ = stack
    c = 256
    y0 = (N - c) // 2
    crop = np.ascontiguousarray(raw.reshape(3, DEPTH, 5, N, N)[:, :, :, y0:y0 + c, y0:y0 + c].reshape(-1, c, c))
    prod, orc = product(crop, cfg, otf, c), fp64(crop, cfg, otf, c)
    pc = compare(prod, orc, c)
    print("\nC2 256^2x64 crop, product vs FP64 oracle:", json.dumps(pc))
    assert bar(pc), pc
    if build_ref.build() is not None:
        rc = compare(reference(crop, cfg, otf, c), orc, c)
        print("C2 256^2x64 crop, reference CUDA build vs FP64 oracle:", json.dumps(rc))
