"""Host logic of runs on several ranks, with two gloo processes on the CPU (no GPU): the
bench's barrier and max / sum over ranks, and the sharding of a batch by scene (scene k on
rank k % world; independent scenes need no exchange), which must partition the batch."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["ABD_ROOT"])
import numpy as np
import torch.distributed as dist
import bench
from adb_gb300 import scene as S
rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo", rank=rank, world_size=world)
bench.dist_barrier(world)
mx = bench.dist_max(float(rank + 1) * 1.5, world)
sm = bench.dist_sum(float(rank + 1), world)
full = S.batched_scenes(n_scenes=9, seed=3, hi=12)
mine = full.scenes_of_rank(rank, world)
ranges = full.scene_ranges()
sizes = [b1 - b0 for k, (b0, b1) in enumerate(ranges) if k % world == rank]
ok = [b1 - b0 for b0, b1 in mine.scene_ranges()] == sizes
# each scene of the shard is the same scene as in the full batch, body for body
b = 0
for k, (b0, b1) in enumerate(ranges):
    if k % world != rank:
        continue
    n = b1 - b0
    ok = ok and np.array_equal(mine.q0[b:b + n], full.q0[b0:b1])
    ok = ok and np.array_equal(mine.body_range(b, b + n).rest, full.body_range(b0, b1).rest)
    b += n
tot = bench.dist_sum(float(mine.n_bodies), world)
print(json.dumps({"rank": rank, "max": mx, "sum": sm, "ok": bool(ok), "bodies_total": tot,
                  "full_bodies": full.n_bodies}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reduce_and_shard_scenes():
    pytest.importorskip("torch")
    port = str(free_port())
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1", MASTER_PORT=port,
                   ABD_ROOT=ROOT, CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=300)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    for r in outs:
        assert r["max"] == 3.0 and r["sum"] == 3.0 and r["ok"]
        assert r["bodies_total"] == r["full_bodies"]
