"""The multi-rank path on CPU (gloo, world size 2), with real work per rank.

MSSP shards by source: each rank runs the oracle's MSSP_CPU::run on its own
slice of one source list (dawn_gb300.shard), the distance rows meet on rank
0 in one gather, and the result must equal a single-rank run of the whole
list.  The bench's whole-job figures (bench.aggregate) are then checked on
the ranks' measured times and edge counts.  No GPU: every rank traverses on
the host and the collectives run over gloo."""

import os
import socket
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _graph_and_sources():
    from dawn_gb300 import gen
    g = gen.rmat(12, 8, seed=3)
    return g, gen.sources(g, 37, seed=5)  # 37: slices of 19 and 18 sources


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path[:0] = [ROOT, os.path.join(ROOT, "gal-dawn_gb300"), os.path.join(ROOT, "oracle")]
    import torch
    import torch.distributed as dist
    import bench
    import oracle as O
    from dawn_gb300 import shard
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, _ = bench.dist_env()
    g, srcs = _graph_and_sources()
    mine = shard.shard(srcs, r, ws)
    edges = 0

    def run(s):
        nonlocal edges
        ref, e, _ = O.mssp(g, s, threads=1)
        edges = e
        return O.hops_ref_to_api(ref, s)

    t0 = time.perf_counter()
    rows = shard.my_rows(srcs, r, ws, run)
    ms = (time.perf_counter() - t0) * 1e3
    full = shard.gather_rows(torch, rows, len(srcs), r, ws)
    out = bench.aggregate(torch, ms, edges, ws, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, ws, mine.tolist(), ms, edges, out, full))


def test_two_ranks_shard_and_gather():
    import torch.multiprocessing as mp
    sys.path[:0] = [os.path.join(ROOT, "gal-dawn_gb300"), os.path.join(ROOT, "oracle")]
    import oracle as O
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=180) for _ in procs), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ws0, s0, ms0, e0, out0, full0), (r1, ws1, s1, ms1, e1, out1, full1) = res
    assert (r0, r1, ws0, ws1) == (0, 1, 2, 2)
    g, srcs = _graph_and_sources()
    # contiguous slices covering the list once
    assert s0 + s1 == srcs.tolist() and (len(s0), len(s1)) == (19, 18)
    # rank 0 holds every row, in source order, equal to one rank doing it all
    ref, edges, _ = O.mssp(g, srcs, threads=1)
    assert full1 is None
    assert full0.shape == (len(srcs), g.n)
    assert np.array_equal(full0, O.hops_ref_to_api(ref, srcs))
    # whole-job figures: the slowest rank's time, every rank's edges
    assert e0 + e1 == edges
    for ms, total, gteps in (out0, out1):
        assert ms == max(ms0, ms1) and total == edges
        assert abs(gteps - edges / (ms * 1e-3) / 1e9) < 1e-9


def test_shard_ranges():
    sys.path[:0] = [os.path.join(ROOT, "gal-dawn_gb300")]
    from dawn_gb300 import shard
    for nsrc in (0, 1, 5, 64, 65, 4096):
        for world in (1, 2, 3, 8):
            spans = [shard.shard_range(nsrc, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == nsrc
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [hi - lo for lo, hi in spans]
            assert max(sizes) - min(sizes) <= 1


def test_single_rank_is_identity():
    sys.path[:0] = [ROOT, os.path.join(ROOT, "gal-dawn_gb300")]
    import torch
    import bench
    from dawn_gb300 import shard
    ms, total, gteps = bench.aggregate(torch, 1.5, 600, 1, "cpu")
    assert (ms, total) == (1.5, 600) and abs(gteps - 600 / 1.5e-3 / 1e9) < 1e-12
    rows = np.arange(12, dtype=np.int32).reshape(3, 4)
    assert shard.gather_rows(torch, rows, 3, 0, 1) is rows or np.array_equal(
        shard.gather_rows(torch, rows, 3, 0, 1), rows)
