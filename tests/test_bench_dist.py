"""The benchmark's multi-rank plumbing on the CPU: two gloo ranks, as
torchrun launches them, agree on the max of the per-rank times and the sum
of the per-rank bodies (replicas: no data exchange)."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, json
sys.path.insert(0, sys.argv[1])
import bench
d = bench.Dist()
d.barrier()
t = d.max(1.5 + d.rank)          # per-rank step time
b = d.sum(1000.0 * (d.rank + 1))  # per-rank bodies
d.barrier()
print(json.dumps({"rank": d.rank, "world": d.world, "max": t, "sum": b}))
d.close()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks():
    pytest.importorskip("torch.distributed")
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            o, e = p.communicate(timeout=120)
        except subprocess.TimeoutExpired:
            p.kill()
            o, e = p.communicate()
        assert p.returncode == 0, e
        outs.append(o.strip().splitlines()[-1])
    import json
    res = [json.loads(o) for o in outs]
    for r in res:
        assert r["world"] == 2
        assert r["max"] == 2.5
        assert r["sum"] == 3000.0
