"""GPU: SRX_tuneFFT measures both FFT paths at every site and length of a
handle's volume, records the faster in the plan cache, and a new process
uses the recorded choices; the volume reconstructed with them equals the one
with the built-in choices to float precision."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SETUP = """
import sys, json; sys.path.insert(0, {root!r})
import numpy as np
import cudasirecon_gb300 as sr
from cudasirecon_gb300 import synthetic as syn
o = syn.Optics()
raw = syn.simulate(128, 128, 16, o, seed=3, n_filaments=10).raw
r = sr.Reconstructor(128, 128, raw.shape[0], syn.config_text(o), syn.ra_otf(o, nx_psf=128, nz_psf=64))
r.set_raw(raw)
"""
TUNE = SETUP + """
print(json.dumps(r.tune_fft(2)))
"""
RUN = SETUP + """
r.load_and_rescale(0, 0); r.set_cur_time(0); r.process()
np.save({out!r}, r.result())
print(json.dumps({{s: sr.fft_plan_choice(s, n) for s, n in {pairs!r}}}))
"""


def py(code, cache):
    env = dict(os.environ, SIMRECON_FFT_PLAN_CACHE=str(cache))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_tuned_plans_are_recorded_and_reused(tmp_path):
    cache = tmp_path / "plans" / "fft.tsv"
    before = tmp_path / "before.npy"
    after = tmp_path / "after.npy"
    sites = ["ingest_x", "ingest_y", "overlap_x", "overlap_y", "crosscorr_rows", "crosscorr_cols"]
    pairs = [(s, 128) for s in sites]
    base = py(RUN.format(root=ROOT, out=str(before), pairs=pairs), cache)
    assert all(v[1] == "built-in" for v in base.values())
    report = py(TUNE.format(root=ROOT), cache)
    tuned = {(e["site"], e["n"]): e for e in report["sites"]}
    for p in pairs:  # every site of a 128^2 volume with both paths was measured
        assert p in tuned, (p, sorted(tuned))
        assert tuned[p]["register_ms"] > 0 and tuned[p]["stockham_ms"] > 0
    assert cache.exists() and len(cache.read_text().strip().splitlines()) >= len(pairs)
    got = py(RUN.format(root=ROOT, out=str(after), pairs=pairs), cache)  # a new process
    for s, n in pairs:
        assert got[s] == [tuned[(s, n)]["choice"] == "register", "tuned"]
    a, b = np.load(after), np.load(before)
    assert float(np.linalg.norm(a - b) / np.linalg.norm(b)) < 2e-6
