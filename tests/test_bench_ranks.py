"""bench.py under torchrun with N > 1: the replicas' host-side gloo group
(world size 2 on CPU).  Every rank must see the slowest rank's time, and a
barrier must hold the fast rank until the slow one arrives."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

CHILD = r"""
import json, os, sys, time
sys.path.insert(0, os.environ["BENCH_ROOT"])
import bench
r = bench.Ranks()
assert r.world == 2 and r.dist is not None
t0 = time.perf_counter()
if r.rank == 1:
    time.sleep(0.5)
r.barrier()
waited = time.perf_counter() - t0
mx = r.max(1.5 + r.rank)
r.close()
print(json.dumps({"rank": r.rank, "max": mx, "waited": waited}))
"""


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_ranks_barrier_and_max_gloo_world2():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), BENCH_ROOT=str(ROOT))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    by_rank = {o["rank"]: o for o in outs}
    assert set(by_rank) == {0, 1}
    for o in outs:
        assert o["max"] == 2.5
    # rank 0 reached the barrier first and waited for rank 1's sleep
    assert by_rank[0]["waited"] >= 0.4


def test_ranks_single_process_is_noop(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    r = bench.Ranks()
    assert r.dist is None
    r.barrier()
    assert r.max(3.25) == 3.25
    r.close()
