"""SRX_server*: concurrent requests of several shapes and configurations give
the same volumes as the plain per-handle SR_* flow."""
import numpy as np
import pytest

import cudasirecon_gb300 as sr
from golden_cases import load

pytestmark = pytest.mark.gpu

CASES = ["c3d_64", "c3d_96x80", "c2d_128"]


def plain(case):
    raw = case["raw"][0]
    r = sr.Reconstructor(case["nx"], case["ny"], raw.shape[0], case["config"], case["otf"])
    r.set_raw(raw)
    r.load_and_rescale(0, 0)
    r.set_cur_time(0)
    r.process()
    out = r.result().copy()
    r.close()
    return out


@pytest.mark.parametrize("budget", [150e9, 1.0], ids=["roomy", "evict-every-time"])
def test_server_matches_plain(budget):
    cases = {n: load(n)[0] for n in CASES}
    want = {n: plain(c) for n, c in cases.items()}
    srv = sr.Server(workers=3, hbm_budget=budget)
    cfg = {n: srv.add_config(c["config"], c["otf"]) for n, c in cases.items()}
    jobs = []
    for rep in range(3):
        for n, c in cases.items():
            raw = np.ascontiguousarray(c["raw"][0])
            out = np.zeros(want[n].shape, np.float32)
            jobs.append((n, out, srv.submit(cfg[n], raw, out)))
    for n, out, t in jobs:
        lat = srv.wait(t)
        assert lat > 0
        assert np.array_equal(out, want[n]), n
    if budget > 1e9:
        assert srv.device_bytes() > 0  # handles stay pooled for the next requests
    srv.close()


def test_server_reserve_then_serve():
    case, _ = load("c3d_64")
    want = plain(case)
    srv = sr.Server(workers=2)
    cid = srv.add_config(case["config"], case["otf"])
    raw = np.ascontiguousarray(case["raw"][0])
    assert srv.reserve(cid, case["nx"], case["ny"], raw.shape[0], 2) == 2
    held = srv.device_bytes()
    assert held > 0
    outs = [np.zeros(want.shape, np.float32) for _ in range(4)]
    ts = [srv.submit(cid, raw, o) for o in outs]
    for t, o in zip(ts, outs):
        srv.wait(t)
        assert np.array_equal(o, want)
    assert srv.device_bytes() == held  # the reserved handles served every request
    srv.close()


def test_server_rejects_unknown_config():
    case, _ = load("c3d_64")
    srv = sr.Server(workers=1)
    raw = np.ascontiguousarray(case["raw"][0])
    with pytest.raises(sr.SIReconError):
        srv.submit(5, raw, np.zeros(4, np.float32))
    srv.close()
