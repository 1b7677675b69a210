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


@pytest.mark.parametrize("budget", ["roomy", "one-handle"])
def test_server_matches_plain_within_budget(budget):
    """Every result equals the plain flow's, alone or in the mix.  With room
    for only the largest handle, requests of other shapes wait for it to be
    released and idle handles are deleted: the reserved bytes, polled while
    the requests run, never exceed the budget, and the bytes actually held
    never exceed the reserved ones."""
    import threading
    cases = {n: load(n)[0] for n in CASES}
    want = {n: plain(c) for n, c in cases.items()}
    probe = sr.Server(workers=1)
    pcfg = {n: probe.add_config(c["config"], c["otf"]) for n, c in cases.items()}
    planned = {n: probe.planned_bytes(pcfg[n], c["nx"], c["ny"], c["raw"].shape[1]) for n, c in cases.items()}
    probe.close()
    cap = 150e9 if budget == "roomy" else max(planned.values())
    srv = sr.Server(workers=3, hbm_budget=cap)
    cfg = {n: srv.add_config(c["config"], c["otf"]) for n, c in cases.items()}
    seen, stop = [], threading.Event()

    def poll():
        while not stop.is_set():
            seen.append(srv.memory())

    th = threading.Thread(target=poll)
    th.start()
    jobs = []
    try:
        for rep in range(3):
            for n, c in cases.items():
                raw = np.ascontiguousarray(c["raw"][0])
                out = np.zeros(want[n].shape, np.float32)
                jobs.append((n, out, srv.submit(cfg[n], raw, out)))
        for n, out, t in jobs:
            lat = srv.wait(t)
            assert lat > 0
            assert np.array_equal(out, want[n]), n
    finally:
        stop.set()
        th.join()
    assert seen and max(r for r, _ in seen) <= cap
    assert all(h <= r for r, h in seen)
    assert srv.device_bytes() > 0  # handles stay pooled for the next requests
    if budget == "one-handle":
        c = srv.counters()
        assert c["evicted"] > 0 and c["admission_waits"] > 0, c
    srv.close()


def test_server_request_larger_than_budget_fails_cleanly():
    case, _ = load("c3d_64")
    srv = sr.Server(workers=1, hbm_budget=1 << 20)
    cid = srv.add_config(case["config"], case["otf"])
    raw = np.ascontiguousarray(case["raw"][0])
    out = np.zeros((24, 128, 128), np.float32)
    t = srv.submit(cid, raw, out)
    with pytest.raises(sr.SIReconError, match="budget"):
        srv.wait(t)
    assert srv.device_bytes() == 0
    srv.close()


def test_server_second_wait_on_a_ticket_is_an_error():
    case, _ = load("c3d_64")
    want = plain(case)
    srv = sr.Server(workers=1)
    cid = srv.add_config(case["config"], case["otf"])
    raw = np.ascontiguousarray(case["raw"][0])
    out = np.zeros(want.shape, np.float32)
    t = srv.submit(cid, raw, out)
    srv.wait(t)
    with pytest.raises(sr.SIReconError):
        srv.wait(t)
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


def synthetic_case(nx, nz, twod, seed):
    from cudasirecon_gb300 import synthetic as syn
    o = syn.Optics(nphases=3 if twod else 5)
    raw = syn.simulate(nx, nx, nz, o, seed=seed, n_filaments=10).raw
    otf = syn.ra_otf(o, nx_psf=128, nz_psf=64, norders=2 if twod else 3, twod=twod)
    cfg = syn.config_text(o, twod=twod, extra={"wiener": 0.00048828125} if twod else None)
    return {"nx": nx, "ny": nx, "raw": [raw], "config": cfg, "otf": otf}


def test_batch_uneven_matches_plain():
    """SRX_serverRunBatch over a 2D/3D mix of uneven shapes (radix-2, -3 and -5
    line lengths): every item equals the plain flow's volume, whether its
    chunk ran as a single volume or back to back with overlapped copies."""
    cases = {n: load(n)[0] for n in CASES}
    cases["s3d_384x16"] = synthetic_case(384, 16, False, 11)
    cases["s2d_640"] = synthetic_case(640, 1, True, 12)
    want = {n: plain(c) for n, c in cases.items()}
    srv = sr.Server(workers=2)
    cfg = {n: srv.add_config(c["config"], c["otf"]) for n, c in cases.items()}
    items, names = [], []
    # three items of most shapes (one chunk, run back to back with overlapped
    # copies) and one of the 2D 640^2 shape (the single-volume flow)
    for rep in range(3):
        for n, c in cases.items():
            if n == "s2d_640" and rep > 0:
                continue
            items.append((cfg[n], np.ascontiguousarray(c["raw"][0]), np.zeros(want[n].shape, np.float32)))
            names.append(n)
    srv.run_batch(items)
    for n, (_, _, out) in zip(names, items):
        assert np.array_equal(out, want[n]), n
    # an invalid item fails the call before anything runs
    with pytest.raises(sr.SIReconError):
        srv.run_batch([(99, items[0][1], items[0][2])])
    srv.close()


def test_server_k0_reuse_is_a_later_time_point():
    """k0 kept per configuration: the first request searches k0 and the server
    records it; the next request of the configuration is processed like time
    point 1 of a series whose time point 0 fitted that k0 (k0 kept, modamps
    fitted, its own bleach correction)."""
    case, _ = load("c3d_64_ts")
    raw0, raw1 = (np.ascontiguousarray(case["raw"][t]) for t in (0, 1))
    r = sr.Reconstructor(case["nx"], case["ny"], raw0.shape[0], case["config"], case["otf"])
    r.set_ntimes(2)
    want = []
    for t, raw in enumerate((raw0, raw1)):
        r.set_raw(raw)
        r.load_and_rescale(0, 0)
        r.set_cur_time(t)
        r.process()
        want.append(r.result().copy())
        if t == 0:
            k0_t0 = r.fit()[0]
    r.close()
    srv = sr.Server(workers=2)
    cid = srv.add_config(case["config"], case["otf"])
    srv.set_k0_reuse(cid, True)
    assert srv.recorded_k0(cid) is None
    outs = [np.zeros(w.shape, np.float32) for w in want]
    srv.wait(srv.submit(cid, raw0, outs[0]))
    assert np.array_equal(srv.recorded_k0(cid), k0_t0)
    srv.wait(srv.submit(cid, raw1, outs[1]))
    assert np.array_equal(outs[0], want[0])
    assert np.array_equal(outs[1], want[1])
    # reuse off again: the request searches k0 like a standalone volume
    srv.set_k0_reuse(cid, False)
    out = np.zeros(want[1].shape, np.float32)
    srv.wait(srv.submit(cid, raw1, out))
    assert np.array_equal(out, plain({"raw": [raw1], "nx": case["nx"], "ny": case["ny"], "config": case["config"],
                                      "otf": case["otf"]}))
    srv.close()
