"""CPU: the output-header oracle's min/max restatement against the
reference's sequential `if / else if` loop (cudaSirecon.cpp:1676-1680)."""
import numpy as np

from oracle.mrc_header import minmax_else_if


def loop(v):
    mx, mn = np.float32(-np.finfo(np.float32).max), np.float32(np.finfo(np.float32).max)
    for x in v:
        if x > mx:
            mx = x
        elif x < mn:
            mn = x
    return float(mn), float(mx)


def test_minmax_else_if_matches_sequential_loop():
    rng = np.random.default_rng(3)
    cases = [rng.standard_normal(int(rng.integers(1, 60))).astype(np.float32) for _ in range(300)]
    cases += [np.arange(10, dtype=np.float32), np.arange(10, 0, -1, dtype=np.float32),  # min never set / set
              np.array([5, np.nan, 1, 7, np.nan], np.float32)]
    for v in cases:
        assert minmax_else_if(v) == loop(v), v
