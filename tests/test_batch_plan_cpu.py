"""The uneven-batch schedule (SRX_batchPlan, the plan SRX_serverRunBatch runs),
checked on the CPU: grouping by configuration and shape, chunk sizes, and the
largest-group-first order with each group's chunks together."""
import ctypes as C
from collections import defaultdict

import numpy as np
import pytest

import cudasirecon_gb300 as sr


def plan(items, workers):
    lib = sr.load_library()
    n = len(items)
    arr = (sr.BatchItem * n)()
    for i, (cfg, nx, ny, nimg, u16) in enumerate(items):
        arr[i] = sr.BatchItem(cfg, nx, ny, nimg, 1, int(u16), 1)  # buffers are not touched by the planner
    chunk = (C.c_int * n)()
    nch = lib.SRX_batchPlan(arr, n, workers, chunk)
    assert nch > 0
    return nch, list(chunk)


def test_plan_groups_chunks_and_order():
    rng = np.random.default_rng(6)
    items = [(1, int(s), int(s), 9, True) for s in rng.choice([256, 512, 1024, 2048], 120)]
    items += [(0, 512, 512, 15 * 32, True)] * 3 + [(0, 768, 768, 15 * 64, True)] * 2 + [(0, 256, 256, 15 * 16, False)]
    nch, chunk = plan(items, 6)
    members = defaultdict(list)
    for i, c in enumerate(chunk):
        members[c].append(i)
    assert sorted(members) == list(range(nch))            # every chunk used, every item placed
    for c, idx in members.items():
        assert len({items[i] for i in idx}) == 1           # one configuration, shape and input type
        assert idx == sorted(idx)                          # the caller's order inside a chunk
        assert len(idx) <= 16
    # groups of up to four items are one chunk (one handle, copies overlapped)
    for key in [(0, 512, 512, 480, True), (0, 768, 768, 960, True), (0, 256, 256, 240, False)]:
        assert len({chunk[i] for i, it in enumerate(items) if it == key}) == 1
    # a large group: about one chunk per worker, at most 16 items each
    big = [i for i, it in enumerate(items) if it[1] == 2048]
    per = min(16, max(-(-len(big) // 6), 4))
    assert len({chunk[i] for i in big}) == -(-len(big) // per)
    # execution order: groups by nx * ny * nimages * items, largest first, chunks of a group contiguous
    gkey = {}
    for i, it in enumerate(items):
        gkey.setdefault(chunk[i], it)
    seq = [gkey[c] for c in range(nch)]
    first = {}
    for pos, k in enumerate(seq):
        first.setdefault(k, pos)
    assert all(seq[p] == seq[p - 1] or first[seq[p]] == p for p in range(1, nch))
    cost = {k: k[1] * k[2] * k[3] * sum(1 for it in items if it == k) for k in set(items)}
    order = sorted(first, key=first.get)
    assert [cost[k] for k in order] == sorted((cost[k] for k in order), reverse=True)


def test_plan_single_worker_and_empty_fields():
    nch, chunk = plan([(0, 64, 64, 180, True)] * 20, 1)
    assert nch == 2 and chunk == [0] * 16 + [1] * 4     # at most 16 items per chunk
    nch, chunk = plan([(0, 64, 64, 180, True)], 8)
    assert nch == 1 and chunk == [0]


def test_server_wrapper_rejects_unsupported_inputs_before_the_library():
    """Input checks of the Python server wrapper, made before any library call."""
    srv = sr.Server.__new__(sr.Server)  # no device needed: the checks come first
    srv._keep = {}
    with pytest.raises(ValueError):
        srv.submit(0, np.zeros((15, 8, 8), np.float64), np.zeros(4, np.float32))
    with pytest.raises(ValueError):
        srv.submit(0, np.zeros((15, 8, 8), np.uint16), np.zeros(4, np.float64))
    with pytest.raises(ValueError):
        srv.submit(0, np.zeros((15, 8, 8), np.uint16)[:, ::2], np.zeros(4, np.float32))


def test_uneven_workload_crop_keeps_the_section_order():
    """The uneven benchmark crops one simulated stack to every shape: sections
    stay in Angle -> Z -> Phase order, the crop is centred, and the photon
    level is rescaled about the background."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    ndirs, nph, nz, n = 3, 5, 8, 32
    d, z, p, y, x = np.meshgrid(*[np.arange(k) for k in (ndirs, nz, nph, n, n)], indexing="ij")
    raw = (100 + d * 10000 + z * 1000 + p * 100 + (y * n + x) % 50).astype(np.uint16).reshape(-1, n, n)
    c = bench._crop(raw, ndirs, nph, nz, 16, 4, 1000.0)        # peak 1000: values unchanged
    assert c.shape == (ndirs * 4 * nph, 16, 16) and c.dtype == np.uint16
    want = raw.reshape(ndirs, nz, nph, n, n)[:, 2:6, :, 8:24, 8:24].reshape(-1, 16, 16)
    assert np.array_equal(c, want)
    half = bench._crop(raw, ndirs, nph, nz, 16, 4, 500.0)     # half the photons above the background
    assert np.array_equal(half, np.rint((want.astype(np.float32) - 100) * 0.5 + 100).astype(np.uint16))
