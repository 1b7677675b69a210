"""CPU: the FFT plan cache file (SRX_fftPlanChoice) -- a choice recorded for
this GPU model, site and length overrides the built-in one in a new process;
malformed lines are ignored; lengths without a register path stay Stockham.
Runs in subprocesses with no visible GPU (the model name then reads
"unknown")."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

QUERY = """
import sys; sys.path.insert(0, {root!r})
import cudasirecon_gb300 as sr
for site, n in (("crosscorr_rows", 512), ("crosscorr_rows", 256), ("overlap_x", 128), ("assemble_x", 384)):
    print(site, n, *sr.fft_plan_choice(site, n))
"""


def query(cache):
    env = dict(os.environ, SIMRECON_FFT_PLAN_CACHE=str(cache), CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", QUERY.format(root=ROOT)], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    return {(ln.split()[0], int(ln.split()[1])): (ln.split()[2] == "True", ln.split()[3]) for ln in r.stdout.split("\n")
            if ln.strip()}


def test_plan_cache_overrides_builtin_choice(tmp_path):
    cache = tmp_path / "plans.tsv"
    base = query(cache)  # no file: built-in choices
    assert base[("crosscorr_rows", 512)] == (False, "built-in")
    assert base[("crosscorr_rows", 256)] == (True, "built-in")
    assert base[("assemble_x", 384)] == (False, "stockham-only")
    cache.write_text("unknown\tcrosscorr_rows\t512\tregister\t0.010\t0.012\n"
                     "unknown\tcrosscorr_rows\t256\tstockham\t0.009\t0.008\n"
                     "some other GPU\toverlap_x\t128\tstockham\t1\t0.5\n"
                     "garbage line\n"
                     "unknown\tnot_a_site\t128\tregister\t1\t2\n")
    got = query(cache)
    assert got[("crosscorr_rows", 512)] == (True, "tuned")
    assert got[("crosscorr_rows", 256)] == (False, "tuned")
    assert got[("overlap_x", 128)] == (True, "built-in")  # recorded for another GPU model only
    assert got[("assemble_x", 384)] == (False, "stockham-only")
