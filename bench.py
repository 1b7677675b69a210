#!/usr/bin/env python
"""Benchmark: SIM reconstruction throughput on one GB300.

Workload (default): the time-series configuration -- 512 x 512 px x 48 z x
15 images (3 angles x 5 phases, uint16) per time point, output 1024 x 1024 x
48 float32; k0 is fitted at time 0 (untimed warm-up) and reused for the timed
time points, modamps are re-fitted every time point.  A "step" is one time
point through the whole hot path (ingest -> bleach correction -> band
separation -> modamp fit -> Wiener filter -> assembly).  Metric: output
Mvoxels/s.

  value : steps x output voxels / device time with the raw stack already
          resident in HBM (CUDA events on the library's stream, L2 flushed
          between steps by writing 256 MiB); per-kernel times come from a
          separate profiled pass of the same steps.
  e2e   : the same through the C ABI from pinned host memory with every
          step's upload (377 MB) and download (201 MB) in the timed region:
          SRX_processSeries (copies overlapped with the computation), median
          of three repeats; plain_value is the plain SR_* sequence per volume.

--impl reference runs the reference's own CUDA build (gpuFunctionsImpl.cu +
cuFFT, compiled from the reference sources by oracle/build_ref.py) through
its SR_* flow on the same workload.

--workload uneven: a 2D/3D batch of 560 acquisitions of 28 shapes through
SRX_serverRunBatch vs the plain one-at-a-time flow.  --workload serving:
Poisson arrivals of requests of four configurations through SRX_server*,
p50/p95/p99 latency and throughput vs the plain flow.  --workload makeotf:
SRX_makeOTF on a 128 x 128 x 64 x 5 bead PSF vs the FP64 CPU restatement.
The default line carries compact forms of all three.

Prints one JSON line (rank 0).  N>1 runs independent replicas (one process
per GPU, weak scaling: each rank reconstructs its own time points).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (nx, ny, nz, description)
    "timeseries_512x512x48": (512, 512, 48, "512x512x48x15 uint16 per time point, k0 fitted at t=0 and reused"),
    "plain_256x256x32": (256, 256, 32, "256x256x32x15 uint16 single volume, k0 search on every step"),
}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, world, local, dist
    return rank, world, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def weak_mvox_per_s(world, steps, outvox, seconds):
    """Whole-job throughput of independent replicas: every rank reconstructs
    `steps` volumes of `outvox` output voxels; `seconds` is the max over ranks."""
    return world * steps * outvox / seconds / 1e6


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(nx, ny, nz, nvol, seed=5):
    """Seeded synthetic time points (drift 0.2 px/frame, 1 %/frame bleaching).

    With SIRECON_BENCH_CACHE set to a folder, the stacks are cached there.
    """
    from cudasirecon_gb300 import synthetic as syn
    o = syn.Optics()
    cache = os.environ.get("SIRECON_BENCH_CACHE")
    cpath = os.path.join(cache, f"bench_{nx}x{ny}x{nz}_{nvol}_{seed}.npz") if cache else None
    if cpath and os.path.exists(cpath):
        z = np.load(cpath)
        return [z[f"v{i}"] for i in range(nvol)], z["otf"], str(z["cfg"])
    vols = []
    for t in range(nvol):
        a = syn.simulate(nx, ny, nz, o, seed=seed, drift_px=0.2 * t, bleach=0.99 ** t, noise_seed=1000 + t,
                         scene_seed=seed, mod_seed=seed + 1)
        vols.append(a.raw)
    otf = syn.ra_otf(o, nx_psf=128, nz_psf=64)
    cfg = syn.config_text(o)
    if cpath:
        os.makedirs(cache, exist_ok=True)
        np.savez(cpath, otf=otf, cfg=cfg, **{f"v{i}": v for i, v in enumerate(vols)})
    return vols, otf, cfg


def alg_bytes_per_volume(nx, ny, nz, n_mo, n_red, ndirs=3, nph=5, zoom=2):
    """The measurement's ideal one-pass-per-logical-stage byte count of one
    volume: raw uint16 in, bands out, n_mo overlap builds (3 bands in, 2
    overlaps out), n_red reductions over the overlap pair, bands into the
    filter/assembly, float result out."""
    I, N = ndirs * nph, nx * ny * nz
    hb = (nx // 2 + 1) * ny * nz * 8
    ov = 8 * N
    nout = zoom * zoom * N
    return 2 * I * N + I * hb + n_mo * (3 * hb + 2 * ov) + n_red * 2 * ov + I * hb + 4 * nout


def step_roofline(nx, ny, nz, counts0, counts1, steps, ms_per_step, peak, peak_kind):
    n_mo = (counts1["overlap_builds"] - counts0["overlap_builds"]) / steps
    n_red = (counts1["reductions"] - counts0["reductions"]) / steps
    b = alg_bytes_per_volume(nx, ny, nz, n_mo, n_red)
    ach = b / (ms_per_step / 1e3) / 1e9
    return {"alg_bytes_per_step": int(b), "n_mo": n_mo, "n_red": n_red,
            "k0_searches_per_step": (counts1["k0_searches"] - counts0["k0_searches"]) / steps,
            "achieved": round(ach, 1), "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4),
            "peak_source": peak_kind,
            "what": "whole step: the algorithmic bytes of one volume (raw in, bands, n_mo overlap builds, n_red "
                    "overlap-pair reductions, bands into filter/assembly, result out) over the step time"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_limiter(kernel):
    """The committed full ncu capture's issue-active and DRAM-throughput
    percentages for `kernel` (what bounds it when DRAM is not the limit), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            e = json.load(f).get(kernel)
    except Exception:
        return None
    if not e or "issue_active_pct" not in e:
        return None
    return {k: e[k] for k in ("issue_active_pct", "dram_throughput_pct", "sm_throughput_pct", "full_capture") if k in e}


def ncu_limiter_name(kernel):
    """What bounds `kernel` according to its committed full ncu capture
    ("fp32 issue", "latency", "hbm"), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            e = json.load(f).get(kernel)
    except Exception:
        return None
    return e.get("limiter") if e else None


def ncu_traffic(kernel, workload, alg_bytes_per_launch):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/ncu_traffic.json), or None.  A capture taken on a smaller
    workload is scaled to this launch by its algorithmic bytes (the kernel's
    traffic grows in proportion to the slots it processes)."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            e = json.load(f).get(kernel)
    except Exception:
        return None
    if not e:
        return None
    if e.get("workload") == workload:
        return e["dram_bytes_per_launch"]
    return round(e["dram_bytes_per_launch"] / e["alg_bytes_per_launch"] * alg_bytes_per_launch)


def cpu_baseline(vol, otf, cfg, nx, ny, nz):
    """FP64 oracle on a bounded sample: a 128 x 128 lateral crop of the same stack."""
    import warnings
    from oracle.sirecon_oracle import SIMReconOracle
    c = 128
    crop = vol.reshape(3, nz, 5, ny, nx)[:, :, :, :c, :c].reshape(-1, c, c)
    t = time.perf_counter()
    o = SIMReconOracle(c, c, crop.shape[0], cfg, otf)
    o.set_raw(crop)
    o.load_and_rescale(0)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        o.process()
    dt = time.perf_counter() - t
    outvox = o.result.size
    return {"value": outvox / dt / 1e6, "unit": "Mvoxels/s", "cores": 1, "kind": "port",
            "sample": f"FP64 numpy restatement, full pipeline incl. k0 search, on a {c}x{c}x{nz}x15 lateral crop "
                      f"of the workload ({dt:.1f} s)"}


def run_gb300(args, rank, world, dist, nx, ny, nz, vols, otf, cfg, outvox):
    import cudasirecon_gb300 as sr
    sr.load_library()
    nimg = vols[0].shape[0]
    r = sr.Reconstructor(nx, ny, nimg, cfg, otf)
    r.set_ntimes(1 << 14)
    # time 0: k0 search (untimed)
    r.set_raw(vols[0])
    r.load_and_rescale(0, 0)
    r.set_cur_time(0)
    r.process()
    reuse = args.workload.startswith("timeseries")
    t_idx = 1 if reuse else 0
    # ---- device-resident value
    r.set_raw(vols[1 % len(vols)])
    r.set_cur_time(t_idx)
    r.bench_device(args.warmup)
    l0 = r.kernel_launches()
    fc0 = r.fit_counts()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    barrier(dist)
    dev_ms = r.bench_device(args.steps)
    barrier(dist)
    clk = clocks.stop()
    launches = r.kernel_launches() - l0
    fc1 = r.fit_counts()
    dev_ms = max_over_ranks(dist, dev_ms)
    # per-kernel times from a separate pass of the same steps (the events
    # around every launch would otherwise add to the timed region)
    r.set_profiling(True)
    r.reset_profile()
    prof_ms = r.bench_device(args.steps)
    prof = r.profile()
    r.set_profiling(False)
    value = weak_mvox_per_s(world, args.steps, outvox, dev_ms / 1e3)
    # ---- end to end through the C ABI from page-locked host memory (the
    # library's SRX_hostAlloc buffers; the stacks are copied in before timing)
    host = []
    for v in vols:
        h = sr.host_empty(v.shape, v.dtype)
        h[...] = v
        host.append(h)
    out = sr.host_empty(r.out_shape, np.float32)
    outs2 = [sr.host_empty(r.out_shape, np.float32) for _ in range(2)]
    # (a) the time-series call (SRX_processSeries): volume t's upload and the
    # previous volume's download overlap the computation
    def series(n):
        r.process_series([host[i % len(host)] for i in range(n)], [outs2[i % 2] for i in range(n)], t0=t_idx)
    series(args.warmup)
    # (b) plain per-volume SR_* calls (setRaw -> loadAndRescale -> process -> getResult)
    def plain_one(i):
        r.set_raw(host[i % len(host)])
        r.load_and_rescale(t_idx, 0)
        r.set_cur_time(t_idx)
        r.process()
        r.result(out)

    for i in range(args.warmup):
        plain_one(i)
    # five interleaved repeats of each form, medians reported
    series_s, plain_s, lat = [], [], []
    for rep in range(5):
        barrier(dist)
        t0 = time.perf_counter()
        series(args.steps)
        barrier(dist)
        series_s.append(max_over_ranks(dist, time.perf_counter() - t0))
        barrier(dist)
        t0 = time.perf_counter()
        for i in range(args.steps):
            ts = time.perf_counter()
            plain_one(i)
            lat.append(time.perf_counter() - ts)
        barrier(dist)
        plain_s.append(max_over_ranks(dist, time.perf_counter() - t0))
    e2e_series_s = statistics.median(series_s)
    e2e_s = statistics.median(plain_s)
    # per-volume latency of the plain calls: stack submitted -> result in host memory
    lat_ms = np.sort(np.array(lat)) * 1e3
    latency = {"p50_ms": round(float(np.percentile(lat_ms, 50)), 3), "p99_ms": round(float(np.percentile(lat_ms, 99)), 3),
               "max_ms": round(float(lat_ms[-1]), 3), "n": len(lat),
               "what": "plain SR_* sequence per volume, stack in page-locked host memory -> result in host memory"}
    e2e_plain = weak_mvox_per_s(world, args.steps, outvox, e2e_s)
    # the series numbers its volumes t0, t0+1, ...: for a time-series
    # workload (k0 reused from t = 0) that is the same work as `value`; a
    # workload that searches k0 on every volume keeps the plain path
    e2e = weak_mvox_per_s(world, args.steps, outvox, e2e_series_s if reuse else e2e_s)
    # ---- roofline of the dominant kernel
    kern = prof.get("kernels", {})
    top = max(kern.items(), key=lambda kv: kv[1]["ms"]) if kern else None
    peak, peak_kind = peaks()
    roof = None
    if top:
        name, st = top
        ach = st["alg_bytes"] / (st["ms"] / 1e3) / 1e9
        tr = ncu_traffic(name, args.workload, st["alg_bytes"] / max(1, st["launches"]))
        roof = {"kernel": name, "bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                "limiter": ncu_limiter_name(name),
                "frac": round(ach / peak, 4), "peak_source": peak_kind,
                "traffic": tr, "alg_bytes_per_launch": st["alg_bytes"] / max(1, st["launches"]),
                "avg_launch_ms": st["ms"] / max(1, st["launches"]),
                "share_of_step": round(st["ms"] / max(prof_ms, 1e-9), 4),
                "ncu_full_capture": ncu_limiter(name)}
    line = {
        "metric": "Recon output Mvoxels/s (SIM 3-beam, 512x512x48x15 -> 1024x1024x48)",
        "value": round(value, 1), "unit": "Mvoxels/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded beads+filaments, "
        "widefield PSF, Poisson noise)",
        "config": {"workload": args.workload, "nx": nx, "ny": ny, "nz": nz, "images_per_volume": nimg,
                   "output": list(r.out_shape), "k0": "fitted at t=0, reused" if reuse else "searched every step",
                   "l2": "flushed between steps (256 MiB write); raw stack 377 MB > L2",
                   "timed_volumes": "device value: the t = 1 stack of the drifting, bleaching scene, staged once "
                                    "and reconstructed from the raw stack every step; e2e and plain: the t = 0 "
                                    "and t = 1 stacks alternated",
                   "description": WORKLOADS[args.workload][3]},
        "e2e": {"value": round(e2e, 1), "unit": "Mvoxels/s",
                "h2d_bytes_per_step": int(host[0].nbytes), "d2h_bytes_per_step": int(out.nbytes),
                "api": ("SRX_processSeries (uploads/downloads overlapped with computation), SRX_hostAlloc host buffers"
                        if reuse else "plain SR_* calls per volume (k0 searched on every volume), SRX_hostAlloc host buffers"),
                "plain_value": round(e2e_plain, 1), "plain_latency": latency,
                "repeats_mvox_per_s": {"series": [round(weak_mvox_per_s(world, args.steps, outvox, v), 1) for v in series_s],
                                       "plain": [round(weak_mvox_per_s(world, args.steps, outvox, v), 1) for v in plain_s]},
                "plain_api": "SR_setRawU16 -> SR_loadAndRescaleImage -> SR_processOneVolume -> SR_getResult"},
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": roof,
        "step_roofline": step_roofline(nx, ny, nz, fc0, fc1, args.steps, dev_ms / args.steps, peak, peak_kind),
        "kernels": {k: {"ms_per_step": round(v["ms"] / args.steps, 4), "launches_per_step": v["launches"] / args.steps,
                        "GB_per_s": round(v["alg_bytes"] / (v["ms"] / 1e3) / 1e9, 1) if v["ms"] > 0 else None}
                    for k, v in kern.items()},
        "stages_ms_per_step": {k: round(v["ms"] / args.steps, 4) for k, v in prof.get("stages", {}).items()},
    }
    r.close()
    return line


def run_reference(args, rank, world, dist, nx, ny, nz, vols, otf, cfg, outvox):
    from oracle import build_ref
    lib = build_ref.build()
    if lib is None:
        return {"impl": "reference", "unavailable": "reference CUDA build could not be compiled here"}
    from oracle.refharness import RefRecon
    nimg = vols[0].shape[0]
    fl = [v.astype(np.float32) for v in vols]
    r = RefRecon(nx, ny, nimg, cfg, otf)
    r.set_ntimes(1 << 14)
    r.set_raw(fl[0])
    r.load_and_rescale(0)
    r.set_cur_time(0)
    r.process()
    reuse = args.workload.startswith("timeseries")
    t_idx = 1 if reuse else 0
    out = np.empty(r.out_shape, np.float32)

    def step(i):
        r.set_raw(fl[i % len(fl)])
        r.load_and_rescale(t_idx)
        r.set_cur_time(t_idx)
        r.process()
        out[...] = r.result()

    import ctypes
    ctypes.CDLL(None).fflush(None)
    devnull = os.open(os.devnull, os.O_WRONLY)
    saved = os.dup(1)
    os.dup2(devnull, 1)  # the reference prints progress on stdout
    try:
        for i in range(args.warmup):
            step(i)
        fc0 = r.fit_counts()
        clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
        clocks.start()
        barrier(dist)
        t0 = time.perf_counter()
        for i in range(args.steps):
            step(i)
        barrier(dist)
        dt = max_over_ranks(dist, time.perf_counter() - t0)
        clk = clocks.stop()
        fc1 = r.fit_counts()
    finally:
        import ctypes
        ctypes.CDLL(None).fflush(None)  # flush the reference's C stdio before restoring stdout
        sys.stdout.flush()
        os.dup2(saved, 1)
        os.close(devnull)
    value = world * args.steps * outvox / dt / 1e6
    r.close()
    peak, peak_kind = peaks()
    return {
        "impl": "reference",
        "metric": "Recon output Mvoxels/s (SIM 3-beam, 512x512x48x15 -> 1024x1024x48)",
        "value": round(value, 1), "unit": "Mvoxels/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "nx": nx, "ny": ny, "nz": nz, "images_per_volume": nimg,
                   "k0": "fitted at t=0, reused" if reuse else "searched every step",
                   "timed_volumes": "the same two synthetic time points as the gb300 arm, alternated"},
        "e2e": {"value": round(value, 1), "unit": "Mvoxels/s", "h2d_bytes_per_step": int(fl[0].nbytes),
                "d2h_bytes_per_step": int(out.nbytes),
                "api": "the reference's SR_setRaw (float32 stack) -> loadAndRescaleImage -> processOneVolume -> "
                       "getResult, host memory in and out"},
        "step_roofline": step_roofline(nx, ny, nz, fc0, fc1, args.steps, dt * 1e3 / args.steps, peak, peak_kind),
        "cpu_baseline": {"value": round(value, 1), "unit": "Mvoxels/s", "cores": os.cpu_count(), "kind": "reference",
                         "sample": "the reference's own CUDA build (gpuFunctionsImpl.cu kernels + cuFFT, host "
                                   "orchestration restated from cudaSirecon.cpp, built with OpenMP like the "
                                   "reference) through its SR_* flow on the full workload; deskewOneSection's "
                                   "OpenMP loop uses every host thread, the rest runs on one"},
        "clocks": clk,
    }


# Serving mix: 4 acquisition configurations (two 3D, two 2D, different line
# spacings and pattern angles) with sizes drawn from the time-series and
# uneven-batch shapes; every request is a standalone volume (k0 fitted).
SERVING_CONFIGS = [
    dict(twod=False, ls=0.2035, angles=(-0.8043, -1.8555, 0.2388)),
    dict(twod=False, ls=0.21, angles=(-0.6, -1.647, 0.447)),
    dict(twod=True, ls=0.195, angles=(-0.7, -1.747, 0.347)),
    dict(twod=True, ls=0.22, angles=(-0.9, -1.947, 0.147)),
]
SERVING_SIZES = {False: [(256, 256, 32), (512, 512, 32)], True: [(512, 512, 1), (1024, 1024, 1)]}


def serving_requests(seed=8):
    """One seeded raw volume per (configuration, size) type.  2D configs use
    wiener = 2^-11 (the reference's flag-byte reading of wiener = 0.001 would
    drop every 2D overlap)."""
    from cudasirecon_gb300 import synthetic as syn
    types = []
    cache = os.environ.get("SIRECON_BENCH_CACHE")
    for ci, c in enumerate(SERVING_CONFIGS):
        o = syn.Optics(ls=c["ls"], angles=c["angles"], nphases=3 if c["twod"] else 5)
        otf = syn.ra_otf(o, nx_psf=128, nz_psf=64, norders=2 if c["twod"] else 3, twod=c["twod"])
        cfg = syn.config_text(o, twod=c["twod"], extra={"wiener": 0.00048828125} if c["twod"] else None)
        for (nx, ny, nz) in SERVING_SIZES[c["twod"]]:
            cp = os.path.join(cache, f"serve_{ci}_{nx}x{ny}x{nz}_{seed}.npy") if cache else None
            if cp and os.path.exists(cp):
                raw = np.load(cp)
            else:
                raw = syn.simulate(nx, ny, nz, o, seed=seed + ci, n_filaments=30).raw
                if cp:
                    os.makedirs(cache, exist_ok=True)
                    np.save(cp, raw)
            types.append(dict(config=ci, cfg=cfg, otf=otf, raw=np.ascontiguousarray(raw), nx=nx, ny=ny, nz=nz,
                              outvox=4 * nx * ny * nz))
    return types


def _locked_copy(sr, a):
    """a copied into page-locked host memory from the library (SRX_hostAlloc)."""
    h = sr.host_empty(a.shape, a.dtype)
    h[...] = a
    return h


def run_serving(args, compact=False):
    """Plain one-at-a-time vs served (SRX_server*, Poisson arrivals).
    compact: the summary the default benchmark line carries (100 plain
    requests, one saturated run each with and without k0 kept per
    configuration, Poisson arrivals at 100 req/s)."""
    import threading
    import cudasirecon_gb300 as sr
    sr.load_library()
    types = serving_requests()
    for t in types:  # inputs and result buffers page-locked for both arms
        t["raw"] = _locked_copy(sr, t["raw"])
    rng = np.random.default_rng(8)
    workers = int(os.environ.get("SIRECON_SERVE_WORKERS", "6"))  # 6 measured faster than 4
    # ---- plain: one handle per type, requests one after another
    hs = {}
    for i, t in enumerate(types):
        r = sr.Reconstructor(t["nx"], t["ny"], t["raw"].shape[0], t["cfg"], t["otf"])
        o = sr.host_empty(r.out_shape, np.float32)
        o[...] = 0.0
        hs[i] = (r, o)

    def plain(i):
        r, out = hs[i]
        r.set_raw(types[i]["raw"])
        r.load_and_rescale(0, 0)
        r.set_cur_time(0)
        r.process()
        r.result(out)

    for i in range(len(types)):
        plain(i)
    seq = rng.integers(0, len(types), 100 if compact else 200)
    t0 = time.perf_counter()
    lat = []
    for i in seq:
        ts = time.perf_counter()
        plain(int(i))
        lat.append((time.perf_counter() - ts) * 1e3)
    plain_s = time.perf_counter() - t0
    plain_vox = sum(types[int(i)]["outvox"] for i in seq)
    for r, o in hs.values():
        r.close()
    plain_line = {"requests": len(seq), "req_per_s": round(len(seq) / plain_s, 1),
                  "mvox_per_s": round(plain_vox / plain_s / 1e6, 1),
                  "p50_ms": round(float(np.percentile(lat, 50)), 2), "p99_ms": round(float(np.percentile(lat, 99)), 2)}
    # ---- served
    srv = sr.Server(workers=workers, hbm_budget=150e9)
    cid = {}
    for t in types:
        if t["config"] not in cid:
            cid[t["config"]] = srv.add_config(t["cfg"], t["otf"])
    shapes = [(t["nz"], 2 * t["ny"], 2 * t["nx"]) for t in types]
    for t in types:  # one handle per worker for every shape, created before the timed runs
        srv.reserve(cid[t["config"]], t["nx"], t["ny"], t["raw"].shape[0], workers)
    warm = [np.empty(shapes[i], np.float32) for _ in range(workers) for i in range(len(types))]
    tick = [srv.submit(cid[types[i % len(types)]["config"]], types[i % len(types)]["raw"], warm[i])
            for i in range(len(warm))]
    for k in tick:
        srv.wait(k)
    # result buffers: a pool of 8 per type, page-locked before the timed runs
    # (large device-to-host copies into pageable memory go through the
    # driver's staging buffers, which concurrent workers share); requests of
    # one type share the input, so a buffer written by two requests in flight
    # still ends up with their (identical) result
    pool = [[sr.host_empty(shapes[i], np.float32) for _ in range(8)] for i in range(len(types))]
    for bufs in pool:
        for b in bufs:
            b[...] = 0.0
    dur = float(os.environ.get("SIRECON_SERVE_SECONDS", "2" if compact else "3"))

    def poisson(lams):
        res = []
        for lam in lams:
            n = max(10, int(lam * dur))
            arrivals = np.cumsum(rng.exponential(1.0 / lam, n))
            kinds = rng.integers(0, len(types), n)
            bufs = [pool[int(k)][j % 8] for j, k in enumerate(kinds)]
            tickets = [None] * n
            start = time.perf_counter()

            def submitter():
                for j in range(n):
                    d = start + arrivals[j] - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                    t = types[int(kinds[j])]
                    tickets[j] = srv.submit(cid[t["config"]], t["raw"], bufs[j])

            th = threading.Thread(target=submitter)
            th.start()
            lats = []
            for j in range(n):
                while tickets[j] is None:
                    time.sleep(0.0005)
                lats.append(srv.wait(tickets[j]))
            th.join()
            wall = time.perf_counter() - start
            vox = sum(types[int(k)]["outvox"] for k in kinds)
            res.append({"lambda_req_s": lam, "requests": n, "p50_ms": round(float(np.percentile(lats, 50)), 2),
                        "p95_ms": round(float(np.percentile(lats, 95)), 2),
                        "p99_ms": round(float(np.percentile(lats, 99)), 2),
                        "req_per_s": round(n / wall, 1), "mvox_per_s": round(vox / wall / 1e6, 1)})
        return res

    def saturated_run():
        t0 = time.perf_counter()
        tk = [srv.submit(cid[types[int(i)]["config"]], types[int(i)]["raw"], pool[int(i)][j % 8])
              for j, i in enumerate(seq)]
        lat = [srv.wait(k) for k in tk]
        dt = time.perf_counter() - t0
        return {"requests": len(seq), "req_per_s": round(len(seq) / dt, 1), "mvox_per_s": round(plain_vox / dt / 1e6, 1),
                "p50_ms": round(float(np.percentile(lat, 50)), 2), "p99_ms": round(float(np.percentile(lat, 99)), 2)}

    def set_reuse(on):
        for c in cid.values():
            srv.set_k0_reuse(c, on)
        if on:  # one request per type records each configuration's k0
            for i, t in enumerate(types):
                srv.wait(srv.submit(cid[t["config"]], t["raw"], pool[i][0]))

    # saturated: the plain arm's 200 requests all submitted at once (peak
    # served throughput; latency here is mostly queueing), searching k0 and
    # with k0 kept per configuration, alternated
    sat = {False: [], True: []}
    for on in ((False, True) if compact else (False, True, False, True)):
        set_reuse(on)
        sat[on].append(saturated_run())
    set_reuse(False)
    saturated = max(sat[False], key=lambda d: d["req_per_s"])
    served = poisson((100,) if compact else (5, 20, 50, 100, 200))
    set_reuse(True)
    reuse_saturated = max(sat[True], key=lambda d: d["req_per_s"])
    reuse_served = [] if compact else poisson((20, 100, 200))
    dev = srv.device_bytes()
    srv.close()
    if compact:
        return {"what": "4 acquisition configurations (two 3D 256^2x32 / 512^2x32, two 2D 512^2 / 1024^2), "
                        f"{workers} workers, 150 GB HBM admission budget; every request a standalone volume",
                "plain_req_per_s": plain_line["req_per_s"], "plain_p50_ms": plain_line["p50_ms"],
                "plain_p99_ms": plain_line["p99_ms"],
                "served_saturated_req_per_s": saturated["req_per_s"],
                "served_vs_plain": round(saturated["req_per_s"] / plain_line["req_per_s"], 3),
                "served_k0_kept_saturated_req_per_s": reuse_saturated["req_per_s"],
                "served_k0_kept_vs_plain": round(reuse_saturated["req_per_s"] / plain_line["req_per_s"], 3),
                "poisson_100_req_s": served[0], "handles_bytes": dev}
    return {"metric": "Served recon latency (p50/p95/p99) and throughput vs plain one-at-a-time",
            "unit": "ms / Mvoxels/s", "impl": "gb300", "n_gpus": 1, "data": "synthetic",
            "config": {"workload": "serving",
                       "types": [f"{'2D' if SERVING_CONFIGS[t['config']]['twod'] else '3D'} cfg{t['config']} "
                                 f"{t['nx']}x{t['ny']}x{t['nz']}" for t in types],
                       "workers": workers, "hbm_budget_bytes": 150e9, "handles_bytes": dev,
                       "request": "standalone volume, k0 searched", "arrivals": "Poisson, seeded",
                       "buffers": "raw stacks and result buffers page-locked, SRX_hostAlloc (both arms)"},
            "plain": plain_line, "served_saturated": saturated, "served": served,
            "k0_reuse_per_config": {"served_saturated": reuse_saturated, "served": reuse_served},
            "saturated_repeats_req_per_s": {"search": [d["req_per_s"] for d in sat[False]],
                                            "k0_reuse": [d["req_per_s"] for d in sat[True]]}}


UNEVEN_2D = [256, 512, 1024, 2048]
UNEVEN_3D_XY = [256, 384, 512, 640, 768]
UNEVEN_3D_Z = [16, 24, 32, 48, 64]


def _crop(raw, ndirs, nph, nz, n_xy, nz_new, peak):
    """Centre crop of an Angle->Z->Phase stack to n_xy^2 x nz_new, rescaled
    from the simulated 1000-photon peak (background 100) to `peak`."""
    ny, nx = raw.shape[1:]
    v = raw.reshape(ndirs, nz, nph, ny, nx)
    y0, x0, z0 = (ny - n_xy) // 2, (nx - n_xy) // 2, (nz - nz_new) // 2
    c = v[:, z0:z0 + nz_new, :, y0:y0 + n_xy, x0:x0 + n_xy].astype(np.float32)
    c = (c - 100.0) * (peak / 1000.0) + 100.0
    return np.ascontiguousarray(np.clip(np.rint(c), 0, 65535).astype(np.uint16).reshape(-1, n_xy, n_xy))


def uneven_items(n2d=500, n3d=60):
    """The uneven batch: n2d 2D frames (3 angles x 3 phases, nz = 1) with
    nx = ny drawn from UNEVEN_2D (seed 6) and n3d 3D volumes (3 x 5 images per
    z) with nx = ny drawn from UNEVEN_3D_XY and nz from UNEVEN_3D_Z (seed 7),
    in one seeded random order.  Each shape's stack is a centre crop of one
    simulated acquisition per dimensionality (2048^2 2D, 768^2 x 64 3D), so
    the illumination pattern is the simulated one, rescaled to a peak drawn
    from U[300, 3000] photons for that shape; items of one shape share it."""
    from cudasirecon_gb300 import synthetic as syn
    cache = os.environ.get("SIRECON_BENCH_CACHE")
    r2, r3 = np.random.default_rng(6), np.random.default_rng(7)
    s2 = [int(v) for v in r2.choice(UNEVEN_2D, n2d)]
    s3 = [(int(a), int(b)) for a, b in zip(r3.choice(UNEVEN_3D_XY, n3d), r3.choice(UNEVEN_3D_Z, n3d))]
    cfgs = {}
    for twod in (True, False):
        o = syn.Optics(nphases=3 if twod else 5)
        otf = syn.ra_otf(o, nx_psf=128, nz_psf=64, norders=2 if twod else 3, twod=twod)
        cfg = syn.config_text(o, twod=twod, extra={"wiener": 0.00048828125} if twod else None)
        nx, nz = (2048, 1) if twod else (768, 64)
        cp = os.path.join(cache, f"uneven_master_{'2d' if twod else '3d'}.npy") if cache else None
        if cp and os.path.exists(cp):
            master = np.load(cp)
        else:
            master = syn.simulate(nx, nx, nz, o, seed=6 if twod else 7, n_filaments=50).raw
            if cp:
                os.makedirs(cache, exist_ok=True)
                np.save(cp, master)
        cfgs[twod] = dict(cfg=cfg, otf=otf, master=master, nph=3 if twod else 5, nz=nz)
    stacks = {}
    for key in sorted(set((True, n, 1) for n in s2) | set((False, n, z) for n, z in s3)):
        twod, n, z = key
        c = cfgs[twod]
        peak = float(np.random.default_rng(100000 * twod + 100 * n + z).uniform(300, 3000))
        stacks[key] = _crop(c["master"], 3, c["nph"], c["nz"], n, z, peak)
    order = [(True, n, 1) for n in s2] + [(False, n, z) for n, z in s3]
    perm = np.random.default_rng(6).permutation(len(order))
    return [order[k] for k in perm], stacks, cfgs


MAKEOTF_ARGS = ["-angle", "-0.8043", "-ls", "0.2035", "-xyres", "0.08", "-zres", "0.125", "-na", "1.42",
                "-nimm", "1.515", "-wavelength", "528", "-fixorigin", "3", "20"]


def run_makeotf(args, reps=20):
    """makeotf on the 128 x 128 x 64 x 5 bead PSF the reconstruction's OTF
    is made from: SRX_makeOTF (host PSF in, host OTF array out, everything
    between them on the GPU) against the FP64 numpy restatement of
    radialft.cpp on one host core.  The shipped program's FFTW path does not
    build here (FFTW3f and libtiff are absent)."""
    import cudasirecon_gb300 as sr
    from cudasirecon_gb300.synthetic import Optics, bead_psf_stack
    sr.load_library()
    psf = bead_psf_stack(128, 128, 64, Optics())
    for _ in range(3):
        got = sr.make_otf(psf, MAKEOTF_ARGS)
    times = []
    for _ in range(reps):
        t = time.perf_counter()
        sr.make_otf(psf, MAKEOTF_ARGS)
        times.append(time.perf_counter() - t)
    gpu_ms = statistics.median(times) * 1e3
    from oracle import makeotf_oracle as mo
    t = time.perf_counter()
    want = mo.makeotf(psf, mo.MakeOTFOptions.from_args(MAKEOTF_ARGS))
    cpu_s = time.perf_counter() - t
    g, w = got.astype(np.float64).ravel(), np.asarray(want, np.float64).ravel()
    rel = float(np.linalg.norm(g - w) / max(np.linalg.norm(w), 1e-300))
    return {"psf": "128x128x64x5 float32 bead stack (seeded synthetic), 3 orders, -fixorigin 3 20",
            "ms_per_otf": round(gpu_ms, 3), "ms_per_otf_p95": round(float(np.percentile(times, 95)) * 1e3, 3),
            "reps": reps, "timing": "wall clock around SRX_makeOTF: H2D of the PSF, all kernels, D2H of the OTF",
            "cpu_baseline": {"value_ms_per_otf": round(cpu_s * 1e3, 1), "cores": 1, "kind": "port",
                             "sample": "one full OTF by the FP64 numpy restatement of radialft.cpp"},
            "speedup_vs_cpu": round(cpu_s * 1e3 / gpu_ms, 1), "rel_l2_vs_oracle": rel}


def run_uneven(args, compact=False):
    """C4: the uneven 2D/3D batch, plain one-volume-at-a-time SR_* flow vs
    SRX_serverRunBatch (per-shape chunks, copies overlapped, shapes
    concurrent on the workers' streams).  compact: 100 2D frames and 12 3D
    volumes of the same size distributions (the default line's summary)."""
    import cudasirecon_gb300 as sr
    sr.load_library()
    order, stacks, cfgs = uneven_items(100, 12) if compact else uneven_items()
    stacks = {k: _locked_copy(sr, a) for k, a in stacks.items()}
    outvox = {k: 4 * k[1] * k[1] * k[2] for k in stacks}
    total_vox = sum(outvox[k] for k in order)
    # ---- plain: one handle per shape (created before the timed run)
    hs = {}
    for k, a in stacks.items():
        c = cfgs[k[0]]
        r = sr.Reconstructor(k[1], k[1], a.shape[0], c["cfg"], c["otf"])
        hs[k] = (r, np.full(r.out_shape, 0.0, np.float32))

    def plain(k):
        r, out = hs[k]
        r.set_raw(stacks[k])
        r.load_and_rescale(0, 0)
        r.set_cur_time(0)
        r.process()
        r.result(out)

    for k in stacks:
        plain(k)
    plain_s = []
    for _ in range(1 if compact else 2):
        t0 = time.perf_counter()
        for k in order:
            plain(k)
        plain_s.append(time.perf_counter() - t0)
    want = {k: hs[k][1].copy() for k in stacks}
    for r, _ in hs.values():
        r.close()
    hs.clear()
    # ---- batched
    workers = int(os.environ.get("SIRECON_BATCH_WORKERS", "6"))  # 6 measured faster than 4 and 8
    # the batch's handles (28 shapes, a few per 2D shape) fit in 200 GB of the
    # GPU's 284 GB, so repeated batches reuse them instead of re-creating
    budget = float(os.environ.get("SIRECON_BATCH_BUDGET_GB", "200")) * 1e9
    srv = sr.Server(workers=workers, hbm_budget=budget)
    cid = {twod: srv.add_config(c["cfg"], c["otf"]) for twod, c in cfgs.items()}
    # result buffers: two per shape, touched up front (items of one shape
    # share their input, so every write leaves the same volume)
    pool = {k: [np.full((k[2], 2 * k[1], 2 * k[1]), 0.0, np.float32) for _ in range(2)] for k in stacks}
    items = [(cid[k[0]], stacks[k], pool[k][j % 2]) for j, k in enumerate(order)]
    srv.run_batch(items)  # warm-up: creates the handles of every shape
    warm_counts = srv.counters()
    batch_s = []
    for _ in range(2 if compact else max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        srv.run_batch(items)
        batch_s.append(time.perf_counter() - t0)
    written = {(k, j % 2) for j, k in enumerate(order)}
    same = all(np.array_equal(pool[k][b], want[k]) for k, b in written)
    dev = srv.device_bytes()
    counts = srv.counters()
    timed_counts = {k: counts[k] - warm_counts[k] for k in counts}
    srv.close()
    bs, ps = statistics.median(batch_s), statistics.median(plain_s)
    n2 = sum(1 for k in order if k[0])
    if compact:
        return {"what": f"{n2} 2D frames (256^2-2048^2) and {len(order) - n2} 3D volumes (256^2-768^2, nz 16-64), "
                        "standalone acquisitions, one batch call vs one SR_* flow per item",
                "batched_mvox_per_s": round(total_vox / bs / 1e6, 1), "plain_mvox_per_s": round(total_vox / ps / 1e6, 1),
                "batched_vs_plain": round(ps / bs, 3), "identical_to_plain": bool(same), "shapes": len(stacks)}
    return {"metric": "Recon output Mvoxels/s, uneven 2D/3D batch (batched vs plain)", "impl": "gb300",
            "value": round(total_vox / bs / 1e6, 1), "unit": "Mvoxels/s", "higher_is_better": True, "n_gpus": 1,
            "data": "synthetic", "dtype": "f32",
            "batched_s": [round(v, 3) for v in batch_s], "plain_s": [round(v, 3) for v in plain_s],
            "plain_value": round(total_vox / ps / 1e6, 1), "identical_to_plain": bool(same),
            "config": {"workload": "uneven", "items_2d": n2, "items_3d": len(order) - n2,
                       "shapes": len(stacks), "workers": workers, "hbm_budget_bytes": budget, "handles_bytes": dev,
                       "handles_created_evicted_in_timed_runs": timed_counts,
                       "request": "standalone acquisition, k0 searched",
                       "buffers": "raw stacks page-locked (SRX_hostAlloc), results pageable (both arms)"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=list(WORKLOADS) + ["serving", "uneven", "makeotf"],
                    default="timeseries_512x512x48")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="leave out the serving and uneven-batch summaries of the default line")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local, dist = dist_init()
    if args.impl == "reference" and rank != 0:
        return
    if args.impl == "reference":
        world, dist = 1, None
    if args.workload in ("serving", "uneven", "makeotf"):
        run = {"serving": run_serving, "uneven": run_uneven, "makeotf": run_makeotf}[args.workload]
        if rank == 0 and args.impl != "reference":
            print(json.dumps(run(args)), flush=True)
        elif rank == 0:
            print(json.dumps({"impl": "reference",
                              "unavailable": f"the {args.workload} workload has no reference arm"}))
        return
    nx, ny, nz, _ = WORKLOADS[args.workload]
    vols, otf, cfg = make_workload(nx, ny, nz, 2)
    outvox = 4 * nx * ny * nz
    if args.impl == "reference":
        line = run_reference(args, rank, world, dist, nx, ny, nz, vols, otf, cfg, outvox)
    else:
        line = run_gb300(args, rank, world, dist, nx, ny, nz, vols, otf, cfg, outvox)
        if rank == 0 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(vols[0], otf, cfg, nx, ny, nz)
        if rank == 0 and not args.no_extras and world == 1:
            del vols
            t0 = time.perf_counter()
            line["serving"] = run_serving(args, compact=True)
            line["uneven_batch"] = run_uneven(args, compact=True)
            line["makeotf"] = run_makeotf(args)
            line["extras_wall_s"] = round(time.perf_counter() - t0, 1)
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
