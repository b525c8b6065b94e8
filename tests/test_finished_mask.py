"""The batch's finished mask of the bitset traversal (bs_init in
gal-dawn_gb300/csrc/msbfs.cu), restated on the CPU from oracle distances.

A vertex leaves the pull lists once its visited word equals the batch's
finished mask.  A source without out-edges reaches no vertex but itself, so
its bit is left out of the mask: every other vertex can then finish, and the
vertices that do are exactly those every other source reaches.  With the
bit kept in, no vertex but such a source could ever finish (a batch of all
vertices as sources holds many of them)."""

import numpy as np

import oracle as O
from dawn_gb300 import gen


def visited_words(g, srcs):
    dist, _, _ = O.mssp(g, srcs, threads=1)
    hops = O.hops_ref_to_api(dist, srcs)  # -1 unreachable, 0 at the source
    reached = hops >= 0
    words = np.zeros(g.n, dtype=object)
    for b in range(len(srcs)):
        for v in np.nonzero(reached[b])[0]:
            words[v] |= 1 << b
    return words


def test_sources_without_out_edges_leave_the_mask():
    g = gen.rmat(12, 8, seed=5)
    deg = g.degrees()
    iso = np.nonzero(deg == 0)[0]
    assert len(iso) >= 8
    rng = np.random.default_rng(6)
    srcs = np.concatenate([iso[:8], rng.choice(np.nonzero(deg > 0)[0], 56, replace=False)]).astype(np.int32)
    rng.shuffle(srcs)
    words = visited_words(g, srcs)
    full_all = (1 << len(srcs)) - 1
    full = sum(1 << b for b, s in enumerate(srcs) if deg[s] > 0)
    # the bits of sources without out-edges sit only on the sources themselves
    for b, s in enumerate(srcs):
        if deg[s] == 0:
            holders = [v for v in range(g.n) if (words[v] >> b) & 1]
            assert holders == [s]
    finished_all = [v for v in range(g.n) if words[v] == full_all]
    finished = [v for v in range(g.n) if words[v] == full]
    assert finished_all == []
    # with the mask, a vertex finishes exactly when every other source reached it
    others = [b for b, s in enumerate(srcs) if deg[s] > 0]
    want = [v for v in range(g.n) if all((words[v] >> b) & 1 for b in others) and v not in set(srcs[deg[srcs] == 0])]
    assert finished == want and len(finished) > g.n // 4
