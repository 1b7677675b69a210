"""Precision at the large configuration: 1024 x 1024 px x 64 z x 15 images
(uint16, the seeded synthetic generator of the time-series workload at the
large size), one standalone volume with its k0 search.

Compares the product (CUDA, through the C ABI) with the reference's own CUDA
build (oracle/refharness: gpuFunctionsImpl.cu compiled unmodified) at the full
size, and the product, the reference's CUDA build and the FP64 oracle
(oracle/sirecon_oracle.py) with each other on a lateral crop of the same
stack (--crop px, all z planes; --crop 0 runs the FP64 oracle at the full
size, about 50 GB of host memory and a quarter of an hour): volume rel-L2,
max-abs / peak, k0 in pixels, modamps.  Prints one JSON line.

Not collected by pytest (generating the stack takes minutes).  Run on a GPU
machine after `python -c "import __graft_entry__ as g; g.build()"`:

    python tests/precision_c2.py [--crop 256] [--no-fp64]
"""
import argparse
import json
import os
import sys
import time
import warnings

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

NX = NY = 1024
NZ = 64
DXY = 0.08


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def compare(name_a, a, name_b, b, nx):
    (va, ka, ma), (vb, kb, mb) = a, b
    dk = 1.0 / (nx * DXY)
    return {"pair": f"{name_a} vs {name_b}", "rel_l2": rel_l2(va, vb),
            "max_abs_of_peak": float(np.abs(va - vb).max() / np.abs(vb).max()),
            "k0_px": float(np.abs(np.asarray(ka, np.float64) - np.asarray(kb, np.float64)).max() / dk),
            "modamp": float(np.abs(np.asarray(ma) - np.asarray(mb)).max())}


def run_all(raw, cfg, otf, nx, fp64):
    """product, reference CUDA build and (fp64) the FP64 oracle on one stack"""
    import cudasirecon_gb300 as sr
    from oracle import build_ref
    nimg = raw.shape[0]
    results, times = {}, {}
    t = time.perf_counter()
    r = sr.Reconstructor(nx, nx, nimg, cfg, otf)
    r.set_raw(raw)
    r.load_and_rescale(0, 0)
    r.set_cur_time(0)
    r.process()
    results["product"] = (r.result().copy(), *r.fit())
    r.close()
    times["product_s"] = round(time.perf_counter() - t, 2)
    if build_ref.build() is not None:
        from oracle import refharness
        t = time.perf_counter()
        ref = refharness.RefRecon(nx, nx, nimg, cfg, otf)
        ref.set_raw(raw.astype(np.float32))
        ref.load_and_rescale(0)
        ref.set_cur_time(0)
        ref.process()
        results["reference_cuda"] = (ref.result().copy(), *ref.fit())
        ref.close()
        times["reference_cuda_s"] = round(time.perf_counter() - t, 2)
    if fp64:
        from oracle.sirecon_oracle import SIMReconOracle
        t = time.perf_counter()
        orc = SIMReconOracle(nx, nx, nimg, cfg, otf)
        orc.set_raw(raw)
        orc.load_and_rescale(0)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            orc.process()
        results["fp64_oracle"] = (np.asarray(orc.result, np.float64), np.asarray(orc.k0), np.asarray(orc.amp))
        times["fp64_oracle_s"] = round(time.perf_counter() - t, 1)
    names = list(results)
    pairs = [compare(a, results[a], b, results[b], nx) for i, a in enumerate(names) for b in names[i + 1:]]
    return pairs, times


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--crop", type=int, default=256, help="lateral crop for the FP64 comparison (0: full size)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 oracle")
    args = ap.parse_args()
    from cudasirecon_gb300 import synthetic as syn
    t = time.perf_counter()
    o = syn.Optics()
    raw = syn.simulate(NX, NY, NZ, o, seed=2).raw
    otf = syn.ra_otf(o, nx_psf=128, nz_psf=64)
    cfg = syn.config_text(o)
    gen_s = round(time.perf_counter() - t, 1)
    line = {"workload": f"{NX}x{NY}x{NZ}x15 uint16, one volume, k0 searched", "generate_s": gen_s}
    full_fp64 = not args.no_fp64 and args.crop == 0
    line["full"], line["full_times"] = run_all(raw, cfg, otf, NX, full_fp64)
    if args.crop and not args.no_fp64:
        c = args.crop
        y0 = (NY - c) // 2
        crop = np.ascontiguousarray(raw.reshape(3, NZ, 5, NY, NX)[:, :, :, y0:y0 + c, y0:y0 + c].reshape(-1, c, c))
        line["crop"] = f"{c}x{c}x{NZ}x15 centre crop of the same stack"
        line["crop_comparisons"], line["crop_times"] = run_all(crop, cfg, otf, c, True)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
