"""The queue dealing of the frontier kernels' warp_expand
(gal-dawn_gb300/csrc/dawn_device.cuh), restated on the CPU: a warp task is
`per` queue entries, 32 or the smallest power of two that covers the queue
in one round of the grid, and warp w takes tasks w, w + nw, ...  Every queue
entry must be dealt to exactly one (warp, lane), lanes at or past `per`
stay idle, and a short queue is spread over as many warps as it has
entries."""

import numpy as np
import pytest


def task_size(qn, nw):
    per = 32
    while per > 1 and (per >> 1) * nw >= qn:
        per >>= 1
    return per


def dealt(qn, nw):
    per = task_size(qn, nw)
    out = []
    for w in range(nw):
        base = w * per
        while base < qn:
            lanes = np.arange(32)
            idx = base + lanes
            out.append(idx[(lanes < per) & (idx < qn)])
            base += nw * per
    return per, (np.concatenate(out) if out else np.zeros(0, np.int64))


@pytest.mark.parametrize("nw", [1, 7, 152, 152 * 8 * 6])
@pytest.mark.parametrize("qn_rel", [0, 1, 31, 32, 33, "nw*16", "nw*32-1", "nw*32", "nw*32+1", "nw*100+5"])
def test_every_entry_dealt_once(nw, qn_rel):
    qn = qn_rel if isinstance(qn_rel, int) else eval(qn_rel, {}, {"nw": nw})
    per, idx = dealt(qn, nw)
    assert 1 <= per <= 32 and per & (per - 1) == 0
    assert idx.size == qn
    assert np.array_equal(np.sort(idx), np.arange(qn))


def test_short_queue_uses_many_warps():
    nw = 152 * 8 * 6
    # 64 frontier vertices: one per warp, not two warps of 32
    assert task_size(64, nw) == 1
    # a queue that fills the grid at 32 entries per warp keeps 32
    assert task_size(nw * 32, nw) == 32
    # in between: the smallest power of two covering the queue in one round
    for qn in (nw + 1, 3 * nw, 17 * nw):
        per = task_size(qn, nw)
        assert per * nw >= qn and (per == 1 or (per // 2) * nw < qn)
