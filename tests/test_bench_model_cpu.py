"""CPU: the benchmark's algorithmic-bytes model of one volume (raw in, bands
out, n_mo overlap builds of 3 band volumes in and 2 overlap volumes out, n_red
reductions over the overlap pair, bands into the filter and assembly, float
result out) and the whole-step roofline built from executed counts."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_alg_bytes_time_series_volume():
    # 512 x 512 x 48 x 15 uint16 -> 1024 x 1024 x 48 float, six overlap builds
    # and six reductions (a k0-reusing fit: 3 directions x orders 1, 2)
    n = 512 * 512 * 48
    hb = 257 * 512 * 48 * 8
    want = 2 * 15 * n + 15 * hb + 6 * (3 * hb + 2 * 8 * n) + 6 * 2 * 8 * n + 15 * hb + 4 * 4 * n
    assert bench.alg_bytes_per_volume(512, 512, 48, 6, 6) == want == 5420089344


def test_step_roofline_uses_executed_counts():
    c0 = {"overlap_builds": 10, "reductions": 20, "k0_searches": 3}
    c1 = {"overlap_builds": 10 + 6 * 4, "reductions": 20 + 6 * 4, "k0_searches": 3}
    r = bench.step_roofline(512, 512, 48, c0, c1, 4, 4.0, 6779.7, "measured")
    assert r["n_mo"] == 6 and r["n_red"] == 6 and r["k0_searches_per_step"] == 0
    assert r["alg_bytes_per_step"] == 5420089344
    assert abs(r["achieved"] - 5420089344 / 4e-3 / 1e9) < 0.1
    assert abs(r["frac"] - r["achieved"] / 6779.7) < 1e-4
