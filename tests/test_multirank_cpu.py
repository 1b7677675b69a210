"""The benchmark's multi-GPU form is independent replicas (one process per GPU,
no collective on the data path): ranks meet only at the barriers around the
timed region and in the max over ranks of the elapsed time.  Those helpers
run here as two gloo ranks on the CPU, launched the way torchrun launches
bench.py (RANK / WORLD_SIZE / MASTER_ADDR / MASTER_PORT in the environment)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, sys, time
sys.path.insert(0, sys.argv[1])
import bench
rank, world, local, dist = bench.dist_init()
bench.barrier(dist)
t0 = time.perf_counter()
time.sleep(0.05 * (rank + 1))          # rank 1 is the slower replica
bench.barrier(dist)
elapsed = bench.max_over_ranks(dist, time.perf_counter() - t0)
mine = bench.max_over_ranks(dist, float(rank + 1))
value = bench.weak_mvox_per_s(world, 10, 4 * 512 * 512 * 48, elapsed)
print(json.dumps({"rank": rank, "world": world, "elapsed": elapsed, "max_rank": mine, "value": value}))
dist.destroy_process_group()
"""


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_gloo_ranks_barrier_and_max():
    pytest.importorskip("torch.distributed")
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert [o["rank"] for o in outs] == [0, 1]
    for o in outs:
        assert o["world"] == 2
        assert o["max_rank"] == 2.0                   # the max over ranks reaches every rank
        assert o["elapsed"] >= 0.1                    # the slower replica's time
    assert outs[0]["elapsed"] == outs[1]["elapsed"]
    # whole-job value: both ranks' volumes over the slower rank's time
    assert abs(outs[0]["value"] - 2 * 10 * 4 * 512 * 512 * 48 / outs[0]["elapsed"] / 1e6) < 1e-6 * outs[0]["value"]


def test_weak_value_formula():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.weak_mvox_per_s(1, 100, 50_331_648, 0.5) == pytest.approx(100 * 50_331_648 / 0.5 / 1e6)
    assert bench.weak_mvox_per_s(4, 100, 50_331_648, 0.5) == pytest.approx(4 * bench.weak_mvox_per_s(1, 100, 50_331_648, 0.5))
