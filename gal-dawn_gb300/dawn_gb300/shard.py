"""Source sharding of multi-source traversals across ranks (one GPU each).

MSSP, APSP and closeness are independent per source: the reference loops
over its source list (src/algorithm/gpu/mssp.cu:26-43,
src/algorithm/gpu/apsp.cu:81-100), so the list splits across ranks with no
exchange while the traversals run.  Each rank holds its own replica of the
graph, traverses a contiguous slice of the sources, and the distance rows
meet on rank 0 in one gather at the end.  Nothing here waits on another
rank's kernels.

    rows = my_rows(sources, rank, world, run)      # run(slice) -> (k, n) rows
    full = gather_rows(torch, rows, len(sources), rank, world)  # rank 0: (S, n)
"""

import numpy as np


def shard_range(nsrc, rank, world):
    """[lo, hi) of rank's slice: contiguous, sizes differ by at most one,
    the first nsrc % world ranks one longer."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank outside the world")
    base, extra = divmod(int(nsrc), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard(sources, rank, world):
    lo, hi = shard_range(len(sources), rank, world)
    return np.ascontiguousarray(np.asarray(sources, np.int32)[lo:hi])


def my_rows(sources, rank, world, run):
    """This rank's distance rows: `run` on its slice of the sources."""
    return run(shard(sources, rank, world))


def gather_rows(torch, rows, nsrc, rank, world, group=None):
    """Rank 0 receives every rank's rows in source order, as one (nsrc, n)
    array; other ranks get None.  Slices are padded to the longest one for
    the collective and trimmed after.  With world == 1 the rows return as
    they are."""
    rows = np.ascontiguousarray(rows)
    if world == 1:
        return rows
    import torch.distributed as dist
    n = rows.shape[1]
    longest = shard_range(nsrc, 0, world)
    longest = longest[1] - longest[0]
    pad = np.zeros((longest, n), rows.dtype)
    pad[:rows.shape[0]] = rows
    t = torch.from_numpy(pad)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    parts = [torch.empty_like(t) for _ in range(world)] if rank == 0 else None
    dist.gather(t, parts, dst=0, group=group)
    if rank != 0:
        return None
    out = []
    for r, p in enumerate(parts):
        lo, hi = shard_range(nsrc, r, world)
        out.append(p[:hi - lo].cpu().numpy())
    return np.concatenate(out, axis=0)
