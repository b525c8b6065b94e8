"""The multi-rank host path of bench.py on CPU (gloo, world size 2): every
rank draws its own sources (the path shards by source, no data exchange),
and the whole-job figures are the slowest rank's step time and the edges of
all ranks.  No GPU: the reductions run on the host."""

import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path[:0] = [ROOT, os.path.join(ROOT, "gal-dawn_gb300")]
    import torch
    import torch.distributed as dist
    import bench
    from dawn_gb300 import gen
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, _ = bench.dist_env()
    g = gen.rmat(10, 8, seed=3)
    srcs = bench.rank_sources(g, r)
    # a rank's step time and edges as the bench would measure them
    ms = 2.0 + r
    edges = 1000 * (r + 1)
    out = bench.aggregate(torch, ms, edges, ws, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, ws, list(map(int, srcs)), out))


def test_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ws0, s0, out0), (r1, ws1, s1, out1) = res
    assert (r0, r1, ws0, ws1) == (0, 1, 2, 2)
    assert s0 != s1 and len(s0) == len(s1)  # each rank its own sources
    # slowest rank's time (3.0 ms), all ranks' edges (1000 + 2000)
    for ms, total, gteps in (out0, out1):
        assert ms == 3.0 and total == 3000
        assert abs(gteps - 3000 / 3e-3 / 1e9) < 1e-12


def test_single_rank_is_identity():
    sys.path[:0] = [ROOT]
    import torch
    import bench
    ms, total, gteps = bench.aggregate(torch, 1.5, 600, 1, "cpu")
    assert (ms, total) == (1.5, 600) and abs(gteps - 600 / 1.5e-3 / 1e9) < 1e-12
