"""Multi-rank path on CPU (gloo, world size 2): replicas only.

Each rank solves its own replica (here: one oracle Newton step on its own seeded
state); the benchmark's job time is the max over ranks and its throughput counts
every rank's elements.  No rank exchanges solver data.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    import bench
    from helpers import channel
    from oracle.pyoracle import Oracle
    case, p, y, ac = channel(4, seed=100 + rank)
    o = Oracle(case, p)
    r0 = np.linalg.norm(o.ElmRes(y, ac))
    y1, a1, st, _ = o.newton(y, ac, y, ac)
    r1 = np.linalg.norm(o.ElmRes(y1, a1))
    local_ms = 10.0 * (rank + 1)  # a fixed, rank-dependent "time"
    ms, value = bench.replica_throughput(local_ms, case.nelem, 3)
    out[rank] = (r0, r1, ms, value, case.nelem)
    dist.destroy_process_group()


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(120)
        assert pr.exitcode == 0
    (a0, a1, ms0, v0, E), (b0, b1, ms1, v1, _) = out[0], out[1]
    assert a0 != b0                      # independent replicas (different seeds)
    assert a1 < 0.05 * a0 and b1 < 0.05 * b0
    assert ms0 == ms1 == 20.0            # max over ranks
    assert v0 == v1 == 2 * E * 3 / 0.020
