"""Index arithmetic of the batched min-plus pull (mw_pull in
gal-dawn_gb300/csrc/msssp.cu), restated on the CPU.

A tail row of 64 sources (256 bytes) is read by a group of 64 / S lanes, S
sources per lane (S = 8 in the build, 4 allowed): lane `sub` of a group owns
the 16-byte quads starting at quad_base(sub, q) = 4 sub + q (64 / Q) for
q < Q = S / 4.  Its active sources are four mask bits per quad; after the
pull, its improved sources go back into the 64-bit mask as two 32-bit words
(lo, hi) ORed over the warp.  The live tails of a 32-entry batch are packed
into a stage by their rank among the live lanes, and group g of round r0
reads stage entry r0 + i * groups + g.  The last test runs that whole
sequence for one vertex on random data and compares it with a direct
min-plus over the in-edges."""

import numpy as np
import pytest

BATCH = 64


def layout(S):
    Q = S // 4
    row_lanes = BATCH // S
    groups = 32 // row_lanes
    return Q, row_lanes, groups


def quad_base(sub, q, Q):
    return 4 * sub + q * (BATCH // Q)


@pytest.mark.parametrize("S", [4, 8])
def test_quads_cover_each_source_once_and_stay_in_the_row(S):
    Q, row_lanes, _ = layout(S)
    seen = np.zeros(BATCH, np.int32)
    for sub in range(row_lanes):
        for q in range(Q):
            b = quad_base(sub, q, Q)
            assert b % 4 == 0 and 0 <= b // 4 < 16  # int4 index inside the 256-byte row
            seen[b:b + 4] += 1
    assert (seen == 1).all()


@pytest.mark.parametrize("S", [4, 8])
def test_each_load_instruction_of_a_group_covers_contiguous_bytes(S):
    # quad q of every lane of a group: one instruction; its 16-byte pieces
    # tile 128 (S = 8) or 256 (S = 4) contiguous bytes
    Q, row_lanes, _ = layout(S)
    for q in range(Q):
        starts = sorted(quad_base(sub, q, Q) * 4 for sub in range(row_lanes))
        assert starts == list(range(starts[0], starts[0] + 16 * row_lanes, 16))


def lane_bits(mask, sub, Q):
    """The lane's active sources: four bits per quad, as the kernel takes
    them out of the mask's low or high word."""
    bits = 0
    lo, hi = mask & 0xFFFFFFFF, mask >> 32
    for q in range(Q):
        b = quad_base(sub, q, Q)
        word = hi if b >= 32 else lo
        bits |= ((word >> (b & 31)) & 15) << (4 * q)
    return bits


def place_bits(imp, sub, Q):
    lo = hi = 0
    for q in range(Q):
        b = quad_base(sub, q, Q)
        part = (imp >> (4 * q)) & 15
        if b >= 32:
            hi |= part << (b & 31)
        else:
            lo |= part << b
    return lo, hi


@pytest.mark.parametrize("S", [4, 8])
@pytest.mark.parametrize("seed", range(4))
def test_mask_bits_out_and_back(S, seed):
    Q, row_lanes, _ = layout(S)
    rng = np.random.default_rng(seed)
    for _ in range(200):
        mask = int(rng.integers(0, 2 ** 63)) | (int(rng.integers(0, 2)) << 63)
        lo = hi = 0
        for sub in range(row_lanes):
            bits = lane_bits(mask, sub, Q)
            for q in range(Q):  # bit t of quad q is source quad_base + t
                for t in range(4):
                    assert ((bits >> (4 * q + t)) & 1) == ((mask >> (quad_base(sub, q, Q) + t)) & 1)
            l, h = place_bits(bits, sub, Q)
            lo |= l
            hi |= h
        assert (hi << 32 | lo) == mask


def stage_batch(masks):
    """Live entries (mask != 0) of a 32-entry batch by their rank among the
    live lanes (popc of the lower lanes' ballot bits)."""
    live = [m != 0 for m in masks]
    stage = {}
    for lane, ok in enumerate(live):
        if ok:
            stage[sum(live[:lane])] = lane
    return stage, sum(live)


@pytest.mark.parametrize("S,unroll", [(4, 4), (8, 2), (8, 3)])
def test_rounds_read_every_live_entry_once(S, unroll):
    _, _, groups = layout(S)
    rng = np.random.default_rng(S * 10 + unroll)
    for _ in range(100):
        masks = [int(x) if rng.random() < 0.6 else 0 for x in rng.integers(1, 2 ** 62, 32)]
        stage, cnt = stage_batch(masks)
        assert sorted(stage) == list(range(cnt))
        read = []
        for r0 in range(0, cnt, groups * unroll):
            for i in range(unroll):
                for g in range(groups):
                    r = r0 + i * groups + g
                    if r < cnt:
                        read.append(stage[r])
        assert sorted(read) == [lane for lane, m in enumerate(masks) if m]


@pytest.mark.parametrize("S,unroll", [(8, 3), (4, 4)])
@pytest.mark.parametrize("seed", range(3))
def test_pull_of_one_vertex_matches_direct_min_plus(S, unroll, seed):
    Q, row_lanes, groups = layout(S)
    rng = np.random.default_rng(100 + seed)
    n, indeg = 300, int(rng.integers(1, 150))
    D = rng.integers(0, 1000, (n, BATCH)).astype(np.int64)
    masks = [int(x) if rng.random() < 0.7 else 0 for x in rng.integers(0, 2 ** 63, n)]
    tails = rng.integers(0, n, indeg)
    weights = rng.integers(1, 64, indeg)
    INF = 0x7FFFFFFF
    # direct: for each source s, the min of D[u][s] + w over tails u whose bit s is set
    want = np.full(BATCH, INF, np.int64)
    for u, w in zip(tails, weights):
        for s in range(BATCH):
            if (masks[u] >> s) & 1:
                want[s] = min(want[s], D[u][s] + w)
    # the kernel's order: 32-entry batches, stage, rounds, per-lane minima
    mn = np.full((32, S), INF, np.int64)
    for kb in range(0, indeg, 32):
        cu = [int(tails[k]) if k < indeg else -1 for k in range(kb, kb + 32)]
        cm = [masks[u] if u >= 0 else 0 for u in cu]
        stage, cnt = stage_batch(cm)
        for r0 in range(0, cnt, groups * unroll):
            for i in range(unroll):
                for lane in range(32):
                    g, sub = lane // row_lanes, lane % row_lanes
                    r = r0 + i * groups + g
                    if r >= cnt:
                        continue
                    src_lane = stage[r]
                    u, w = cu[src_lane], int(weights[kb + src_lane])
                    bits = lane_bits(cm[src_lane], sub, Q)
                    for q in range(Q):
                        for t in range(4):
                            if (bits >> (4 * q + t)) & 1:
                                s = quad_base(sub, q, Q) + t
                                mn[lane, 4 * q + t] = min(mn[lane, 4 * q + t], D[u][s] + w)
    # fold the groups (xor steps of row_lanes, 2 row_lanes, ...): group 0 holds the minima
    off = row_lanes
    while off < 32:
        mn = np.minimum(mn, mn[np.arange(32) ^ off])
        off <<= 1
    got = np.full(BATCH, INF, np.int64)
    for sub in range(row_lanes):
        for q in range(Q):
            for t in range(4):
                got[quad_base(sub, q, Q) + t] = mn[sub, 4 * q + t]
    assert np.array_equal(got, want)
