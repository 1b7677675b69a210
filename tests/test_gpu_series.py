"""SRX_processSeries (uploads/downloads overlapped with computation) against
the plain per-volume SR_* sequence and the reference's golden outputs."""
import numpy as np
import pytest

import cudasirecon_gb300 as sr
from golden_cases import load, rel_l2

pytestmark = pytest.mark.gpu


def plain(case):
    raw = case["raw"]
    r = sr.Reconstructor(case["nx"], case["ny"], raw.shape[1], case["config"], case["otf"])
    r.set_ntimes(raw.shape[0])
    outs = []
    for t in range(raw.shape[0]):
        r.set_raw(raw[t])
        r.load_and_rescale(t, 0)
        r.set_cur_time(t)
        r.process()
        outs.append(r.result())
    r.close()
    return np.stack(outs)


@pytest.mark.parametrize("pinned", [False, True])
def test_series_matches_plain_and_reference(pinned):
    case, ref = load("c3d_64_ts")
    raw = np.ascontiguousarray(case["raw"])
    want = plain(case)
    r = sr.Reconstructor(case["nx"], case["ny"], raw.shape[1], case["config"], case["otf"])
    r.set_ntimes(raw.shape[0])
    raws = [np.ascontiguousarray(raw[t]) for t in range(raw.shape[0])]
    outs = [np.zeros(r.out_shape, np.float32) for _ in range(raw.shape[0])]
    if pinned:
        for a in raws + outs:
            sr.pin(a)
    try:
        r.process_series(raws, outs, t0=0)
    finally:
        if pinned:
            for a in raws + outs:
                sr.unpin(a)
    got = np.stack(outs)
    assert np.array_equal(got, want)
    assert rel_l2(got, ref["result"]) < 1e-4
    # getResult after a series returns the last volume
    assert np.array_equal(r.result(), want[-1])
    r.close()


def test_series_odd_length_then_plain_calls():
    """Odd series lengths leave the last result in the second buffer; later
    plain calls and a second series must still be right."""
    case, _ = load("c3d_64")
    raw = np.ascontiguousarray(case["raw"][0])
    r = sr.Reconstructor(case["nx"], case["ny"], raw.shape[0], case["config"], case["otf"])
    r.set_raw(raw)
    r.load_and_rescale(0, 0)
    r.process()
    want = r.result().copy()
    outs = [np.zeros(r.out_shape, np.float32) for _ in range(3)]
    r.process_series([raw, raw, raw], outs, t0=0)
    for o in outs:
        assert np.array_equal(o, want)
    r.set_raw(raw)
    r.load_and_rescale(0, 0)
    r.process()
    assert np.array_equal(r.result(), want)
    outs2 = [np.zeros(r.out_shape, np.float32) for _ in range(2)]
    r.process_series([raw, raw], outs2, t0=0)
    assert np.array_equal(outs2[1], want)
    r.close()


def test_series_rejects_mismatched_lists():
    case, _ = load("c3d_64")
    raw = np.ascontiguousarray(case["raw"][0])
    r = sr.Reconstructor(case["nx"], case["ny"], raw.shape[0], case["config"], case["otf"])
    with pytest.raises(ValueError):
        r.process_series([raw, raw], [np.zeros(r.out_shape, np.float32)])
    r.close()


@pytest.mark.parametrize("t0", [0, 1])
def test_series_graph_replays_match_plain(t0):
    """Volumes whose fit needs no host decision (k0 reused from t = 0) run as
    a captured CUDA graph per raw/output buffer pair, replayed from the third
    such volume on.  Seven volumes cycling the fixture's two time points:
    every result, and the fitted amplitudes after the series, must equal the
    plain per-volume calls bit for bit."""
    case, _ = load("c3d_64_ts")
    raws = [np.ascontiguousarray(case["raw"][t]) for t in range(case["raw"].shape[0])]
    n = 7
    seq = [raws[i % len(raws)] for i in range(n)]
    r = sr.Reconstructor(case["nx"], case["ny"], seq[0].shape[0], case["config"], case["otf"])
    r.set_ntimes(64)
    if t0 > 0:  # k0 of time 0 first, then a series starting at t0
        r.set_raw(seq[0])
        r.load_and_rescale(0, 0)
        r.set_cur_time(0)
        r.process()
    want, want_fit = [], None
    for i in range(n):
        r.set_raw(seq[i])
        r.load_and_rescale(t0 + i, 0)
        r.set_cur_time(t0 + i)
        r.process()
        want.append(r.result().copy())
    want_fit = r.fit()
    outs = [np.zeros(r.out_shape, np.float32) for _ in range(n)]
    l0 = r.kernel_launches()
    r.process_series(seq, outs, t0=t0)
    assert r.kernel_launches() > l0
    for i in range(n):
        assert np.array_equal(outs[i], want[i]), f"volume {i} differs"
    k0, amp = r.fit()
    assert np.array_equal(k0, want_fit[0]) and np.array_equal(amp, want_fit[1])
    # a second call re-captures (options may change between calls) and agrees
    outs2 = [np.zeros(r.out_shape, np.float32) for _ in range(n)]
    r.process_series(seq, outs2, t0=t0)
    for i in range(n):
        assert np.array_equal(outs2[i], want[i])
    r.close()
