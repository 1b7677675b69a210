"""Option coverage against the reference's own CUDA build run live on the GPU
(oracle/refharness: gpuFunctionsImpl.cu compiled unmodified, the config keys
parsed with the reference's storage semantics): bleach-correction modes,
per-time-point k0 search, forced modulation amplitudes, overlap filtering,
order-0 damping off, the fastSI section order and
per-angle OTFs, each on the 64 x 64 x 12 fixture (two time points where the
option concerns time series).  Tolerances: the parity bar."""
import numpy as np
import pytest

import cudasirecon_gb300 as sr
from golden_cases import DXY, load, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refmod():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("the reference CUDA build could not be compiled")
    from oracle import refharness
    return refharness


def run_both(refmod, raws, cfg, otf, nx, ny):
    nt, nimg = raws.shape[:2]
    ref = refmod.RefRecon(nx, ny, nimg, cfg, otf)
    ref.set_ntimes(nt)
    r = sr.Reconstructor(nx, ny, nimg, cfg, otf)
    r.set_ntimes(nt)
    out = []
    for t in range(nt):
        ref.set_raw(raws[t].astype(np.float32))
        ref.load_and_rescale(t)
        ref.set_cur_time(t)
        ref.process()
        r.set_raw(np.ascontiguousarray(raws[t]))
        r.load_and_rescale(t, 0)
        r.set_cur_time(t)
        r.process()
        out.append((r.result().copy(), ref.result().copy(), r.fit(), ref.fit()))
    ref.close()
    r.close()
    return out


def check(out, nx):
    dk = 1.0 / (nx * DXY)
    for got, want, (k0, amp), (rk0, ramp) in out:
        assert np.isfinite(got).all()
        assert rel_l2(got, want) < 1e-4
        assert np.abs(got - want).max() / np.abs(want).max() < 1e-3
        assert np.abs(np.asarray(k0) - np.asarray(rk0)).max() / dk < 1e-3
        assert np.abs(np.asarray(amp) - np.asarray(ramp)).max() < 1e-3


VARIANTS = {
    "equalizez": ("c3d_64", "equalizez=1"),
    "equalizet": ("c3d_64_ts", "equalizet=1"),
    "k0searchAll": ("c3d_64_ts", "k0searchAll=0"),
    "forcemodamp": ("c3d_64", "forcemodamp=0.95"),
    "nofilterovlps": ("c3d_64", "nofilterovlps=0"),
    "dampenOrder0_off": ("c3d_64", "dampenOrder0=0"),
}


@pytest.mark.parametrize("name", list(VARIANTS))
def test_option_matches_reference(refmod, name):
    fixture, extra = VARIANTS[name]
    case, _ = load(fixture)
    cfg = "\n".join(l for l in case["config"].splitlines() if not l.startswith(extra.split("=")[0] + "="))
    cfg += "\n" + extra + "\n"
    check(run_both(refmod, case["raw"], cfg, case["otf"], case["nx"], case["ny"]), case["nx"])


def test_fastsi_order_matches_reference_and_default_order(refmod):
    """Z -> Angle -> Phase sections (fastSI) give what Angle -> Z -> Phase gives."""
    case, _ = load("c3d_64")
    raw = case["raw"][0]
    nz = raw.shape[0] // 15
    fast = raw.reshape(3, nz, 5, *raw.shape[1:]).transpose(1, 0, 2, 3, 4).reshape(raw.shape)[None]
    out = run_both(refmod, fast, case["config"] + "\nfastSI=1\n", case["otf"], case["nx"], case["ny"])
    check(out, case["nx"])
    plain = run_both(refmod, case["raw"], case["config"], case["otf"], case["nx"], case["ny"])
    assert rel_l2(out[0][0], plain[0][0]) < 1e-5


def test_per_angle_otfs_match_reference(refmod):
    """otfPerAngle with one OTF per direction (here the same one three times):
    the same as the shared OTF, and as the reference."""
    case, _ = load("c3d_64")
    otf3 = np.concatenate([case["otf"]] * 3, axis=0)
    out = run_both(refmod, case["raw"], case["config"] + "\notfPerAngle=1\n", otf3, case["nx"], case["ny"])
    check(out, case["nx"])
    plain = run_both(refmod, case["raw"], case["config"], case["otf"], case["nx"], case["ny"])
    assert rel_l2(out[0][0], plain[0][0]) < 1e-6


def test_fewer_output_orders_than_phases_is_refused():
    """nordersout below nphases / 2 + 1 is refused: the reference's separate
    swaps nphases band pointers out of a (2 * norders - 1)-entry vector
    (gpuFunctionsImpl.cu:221-259) and its 3D k0 fit then reads the order-2
    bands (gpuFunctionsImpl.cu:315-324), i.e. memory it never wrote."""
    case, _ = load("c3d_64")
    with pytest.raises(sr.SIReconError, match="nphases must equal 2"):
        sr.Reconstructor(case["nx"], case["ny"], case["raw"].shape[1], case["config"] + "\nnordersout=2\n",
                         case["otf"])
