"""Index arithmetic of the batched min-plus set-up and write-out kernels
(gal-dawn_gb300/csrc/msssp.cu), restated on the CPU.

mw_emit: a warp reads the 32 consecutive 64-word rows of its vertex block
as 512 16-byte pieces (piece p = row p // 16, words 4 (p % 16) .. +3), lays
them into a shared tile with a pitch of 65 words, and lane l reads column c
at word 65 l + c.  mw_init: for source b, every entry k of the source row
lowers the neighbour's word to -(k + 1) with atomicMin, and the entry whose
marker survived stores its weight, so the last entry of a repeated
neighbour wins (the reference CPU path's rule, src/algorithm/cpu/sssp.cpp:
41-46)."""

import numpy as np
import pytest

BATCH, PITCH = 64, 65


@pytest.mark.parametrize("rows", [1, 7, 31, 32])
def test_emit_pieces_cover_each_word_once(rows):
    seen = np.zeros((32, BATCH), np.int32)
    for i in range(32 * BATCH // 4 // 32):
        for lane in range(32):
            p = i * 32 + lane
            r, w0 = p // (BATCH // 4), (p % (BATCH // 4)) * 4
            if r < rows:
                seen[r, w0:w0 + 4] += 1
    assert (seen[:rows] == 1).all() and (seen[rows:] == 0).all()


def test_emit_column_reads_hit_32_banks():
    for c in range(BATCH):
        banks = {(lane * PITCH + c) % 32 for lane in range(32)}
        assert len(banks) == 32


def test_emit_tile_fits_and_pieces_stay_in_the_tile():
    last_piece = 32 * BATCH // 4 - 1
    r, w0 = last_piece // 16, (last_piece % 16) * 4
    assert r * PITCH + w0 + 3 < 32 * PITCH


def init_markers(cols, weights, n, inf=0x7FFFFFFF):
    d = np.full(n, inf, np.int64)
    for k, u in enumerate(cols):            # phase 1: atomicMin of -(k + 1)
        d[u] = min(d[u], -(k + 1))
    for k, u in enumerate(cols):            # phase 2, in any order: the survivor writes
        if d[u] == -(k + 1):
            d[u] = weights[k]
    return d


@pytest.mark.parametrize("seed", range(5))
def test_init_marker_last_entry_wins(seed):
    rng = np.random.default_rng(seed)
    n = 50
    cols = rng.integers(0, n, 200)
    weights = rng.integers(0, 64, 200)
    want = {}
    for k, u in enumerate(cols):            # the reference rule: the last entry wins
        want[int(u)] = int(weights[k])
    got = init_markers(cols, weights, n)
    for u in range(n):
        assert got[u] == want.get(u, 0x7FFFFFFF)
    # the second pass in reverse order gives the same words: once a weight
    # (>= 0) is stored, no marker (< 0) compares equal to it
    d = np.full(n, 0x7FFFFFFF, np.int64)
    for k, u in enumerate(cols):
        d[u] = min(d[u], -(k + 1))
    for k in reversed(range(len(cols))):
        if d[cols[k]] == -(k + 1):
            d[cols[k]] = weights[k]
    assert np.array_equal(d, got)


def test_sparse_segment_relaxes_every_edge_source_pair_once():
    # relax_seg_sparse (mw_push): the lanes take 32 consecutive edges of the
    # segment at a time and walk the vertex's active sources in bit order;
    # every (edge, active source) pair is relaxed once, and each lane's
    # improved sources reach the target's mask in one OR
    rng = np.random.default_rng(9)
    for _ in range(50):
        k0 = int(rng.integers(0, 1000))
        k1 = k0 + int(rng.integers(1, 129))  # a segment holds at most 128 entries
        mask = 0
        for s in rng.choice(64, int(rng.integers(1, 9)), replace=False):
            mask |= 1 << int(s)
        seen = {}
        for kb in range(k0, k1, 32):
            for lane in range(32):
                k = kb + lane
                if k >= k1:
                    continue
                m = mask
                while m:
                    src = (m & -m).bit_length() - 1
                    m &= m - 1
                    seen[(k, src)] = seen.get((k, src), 0) + 1
        want = {(k, s) for k in range(k0, k1) for s in range(64) if (mask >> s) & 1}
        assert set(seen) == want and set(seen.values()) == {1}
