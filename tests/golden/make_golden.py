"""Generate the golden fixtures that pin the oracle and the GPU product.

Two steps:

  python tests/golden/make_golden.py inputs
      (any host) writes tests/golden/in_<case>.npz: seeded synthetic raw
      stacks (uint16), rotationally averaged OTF pages and the config text.

  python tests/golden/make_golden.py outputs --out DIR
      (GB300 host) runs the reference's OWN CUDA kernels through
      oracle/ref_harness on every input and writes DIR/out_<case>.npz with the
      reconstructed volume(s), the fitted k0 / modamps and, for the staged
      case, the separated and the filtered bands of direction 0.  It also
      prints how far the FP64 oracle is from each reference output.

The committed in_*/out_* files are the fixtures; this script is how they
were made.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cudasirecon_gb300 import synthetic as syn  # noqa: E402

CASES = ["c3d_64", "c3d_96x80", "c2d_128", "c2d_128_q", "c3d_64_ts", "c3d_64_w"]


def make_inputs():
    o = syn.Optics()
    # c3d_64: default 3D path, dampenOrder0, staged capture
    a = syn.simulate(64, 64, 12, o, seed=1)
    otf = syn.ra_otf(o, nx_psf=64, nz_psf=24)
    np.savez_compressed(os.path.join(HERE, "in_c3d_64.npz"), raw=a.raw[None], otf=otf,
                        config=syn.config_text(o), nx=64, ny=64, staged=1)
    # c3d_96x80: non-square, radix-3/5 sizes, fastSI section order, equalizez, order-0 suppression
    a = syn.simulate(96, 80, 10, o, seed=11)
    nd, nph = 3, 5
    raw = a.raw.reshape(nd, 10, nph, 80, 96).transpose(1, 0, 2, 3, 4).reshape(-1, 80, 96)
    otf = syn.ra_otf(o, nx_psf=96, nz_psf=20)
    cfg = syn.config_text(o, extra={"fastSI": 1, "equalizez": 1, "wiener": 0.002})
    cfg = cfg.replace("dampenOrder0=1\n", "")
    np.savez_compressed(os.path.join(HERE, "in_c3d_96x80.npz"), raw=raw[None], otf=otf, config=cfg,
                        nx=96, ny=80, staged=1)
    # c2d_128: 2D SIM, 3 dirs x 3 phases, 2D OTF
    o2 = syn.Optics(nphases=3)
    a = syn.simulate(128, 128, 1, o2, seed=21)
    otf = syn.ra_otf(o2, nx_psf=128, norders=2, twod=True)
    # wiener = 2^-11: the low half of its bit pattern is zero, so the reference's
    # int-sized read of bNoKz0 (gpuFunctionsImpl.cu:564) stays false and 2D works
    np.savez_compressed(os.path.join(HERE, "in_c2d_128.npz"), raw=a.raw[None], otf=otf,
                        config=syn.config_text(o2, twod=True, extra={"wiener": 0.00048828125}), nx=128, ny=128,
                        staged=0)
    # wiener = 0.001: the same read turns bNoKz0 on; in 2D every overlap lies in
    # kz = 0, so the reference's fit and output are NaN
    np.savez_compressed(os.path.join(HERE, "in_c2d_128_q.npz"), raw=a.raw[None], otf=otf,
                        config=syn.config_text(o2, twod=True), nx=128, ny=128, staged=0)
    # c3d_64_ts: two time points, k0 fitted at t=0 and reused, bleach correction over time
    a0 = syn.simulate(64, 64, 12, o, seed=1)
    a1 = syn.simulate(64, 64, 12, o, seed=1, drift_px=0.2, bleach=0.99, noise_seed=99)
    otf = syn.ra_otf(o, nx_psf=64, nz_psf=24)
    np.savez_compressed(os.path.join(HERE, "in_c3d_64_ts.npz"), raw=np.stack([a0.raw, a1.raw]), otf=otf,
                        config=syn.config_text(o, extra={"equalizet": 1}), nx=64, ny=64, staged=0)
    # c3d_64_w: kz=0 kept (wiener = 2^-10), no singularity suppression, no order-0 damping
    a = syn.simulate(64, 64, 16, o, seed=31)
    otf = syn.ra_otf(o, nx_psf=64, nz_psf=32)
    cfg = syn.config_text(o, extra={"wiener": 0.0009765625, "nosuppress": 0}).replace("dampenOrder0=1\n", "")
    np.savez_compressed(os.path.join(HERE, "in_c3d_64_w.npz"), raw=a.raw[None], otf=otf, config=cfg,
                        nx=64, ny=64, staged=1)


def load_case(name):
    z = np.load(os.path.join(HERE, f"in_{name}.npz"))
    return dict(raw=z["raw"], otf=z["otf"], config=str(z["config"]), nx=int(z["nx"]), ny=int(z["ny"]),
                staged=int(z["staged"]))


def run_reference(case):
    from oracle.refharness import RefRecon
    raw, nt = case["raw"], case["raw"].shape[0]
    r = RefRecon(case["nx"], case["ny"], raw.shape[1], case["config"], case["otf"])
    res = {}
    if nt > 1:
        r.set_ntimes(nt)
    outs, k0s, amps = [], [], []
    for t in range(nt):
        r.set_raw(raw[t].astype(np.float32))
        r.load_and_rescale(t)
        r.set_cur_time(t)
        if case["staged"]:
            r.stage_separate()
            res["sep_bands_dir0"] = np.stack([r.band(0, b) for b in range(5)]).astype(np.complex64)
            r.stage_fit()
            r.stage_assemble()
            res["filt_bands_dir0"] = np.stack([r.band(0, b) for b in range(5)]).astype(np.complex64)
        else:
            r.process()
        outs.append(r.result())
        k0, amp = r.fit()
        k0s.append(k0)
        amps.append(amp)
    res["result"] = np.stack(outs)
    res["k0"] = np.stack(k0s)
    res["amp"] = np.stack(amps)
    res["k0guess"] = r.k0guess()
    r.close()
    return res


def run_oracle(case):
    from oracle.sirecon_oracle import SIMReconOracle
    raw, nt = case["raw"], case["raw"].shape[0]
    o = SIMReconOracle(case["nx"], case["ny"], raw.shape[1], case["config"], case["otf"])
    o.ntimes = nt
    outs, k0s, amps = [], [], []
    for t in range(nt):
        o.set_raw(raw[t])
        o.load_and_rescale(t)
        o.set_cur_time(t)
        o.process()
        outs.append(o.result)
        k0s.append(o.k0.copy())
        amps.append(o.amp.copy())
    return dict(result=np.stack(outs), k0=np.stack(k0s), amp=np.stack(amps))


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def make_outputs(outdir):
    os.makedirs(outdir, exist_ok=True)
    for name in CASES:
        case = load_case(name)
        t = time.time()
        ref = run_reference(case)
        tr = time.time() - t
        np.savez_compressed(os.path.join(outdir, f"out_{name}.npz"), **ref)
        t = time.time()
        orc = run_oracle(case)
        to = time.time() - t
        dxy = 0.08
        nx = case["nx"]
        dk = 1.0 / (nx * dxy)
        print(f"{name}: ref {tr:.2f}s oracle {to:.2f}s  relL2(vol)={rel_l2(orc['result'], ref['result']):.3e} "
              f"max|dk0|px={np.abs(orc['k0'] - ref['k0']).max() / dk:.3e} "
              f"max|damp|={np.abs(orc['amp'] - ref['amp']).max():.3e}", flush=True)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["inputs", "outputs"])
    ap.add_argument("--out", default=HERE)
    a = ap.parse_args()
    if a.what == "inputs":
        make_inputs()
    else:
        make_outputs(a.out)
