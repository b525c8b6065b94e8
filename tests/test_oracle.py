"""The oracle pinned: hand-computed graphs, the committed golden fixtures
(made by running the reference's own tools), and - where the reference was
compiled here - the reference itself on seeded random graphs."""

import numpy as np
import pytest

import oracle as O
from dawn_gb300 import gen

FLT_MAX = np.float32(3.4028235e38)


class Csr:
    def __init__(self, n, edges, weights=None):
        edges = sorted(edges) if weights is None else None
        self.n = n
        if weights is None:
            src = np.array([e[0] for e in edges], np.int32)
            dst = np.array([e[1] for e in edges], np.int32)
        else:
            order = sorted(range(len(weights)), key=lambda i: weights[i][:2])
            src = np.array([weights[i][0] for i in order], np.int32)
            dst = np.array([weights[i][1] for i in order], np.int32)
            self.w_f32 = np.array([weights[i][2] for i in order], np.float32)
        self.row_ptr = np.zeros(n + 1, np.int32)
        np.add.at(self.row_ptr, src + 1, 1)
        self.row_ptr = np.cumsum(self.row_ptr).astype(np.int32)
        self.col = dst
        self.m = len(dst)


def test_path_and_cycle_hops():
    # 0 -> 1 -> 2 -> 3, 3 -> 0 (directed cycle), 4 isolated
    g = Csr(5, [(0, 1), (1, 2), (2, 3), (3, 0)])
    d, e = O.bfs_queue(g, 0)
    assert d.tolist() == [0, 1, 2, 3, 0]
    assert e == 4
    assert O.bfs_bitmap(g, 0).tolist() == [0, 1, 2, 3, 0]
    d, _ = O.bfs_queue(g, 2)
    assert d.tolist() == [2, 3, 0, 1, 0]
    api = O.hops_ref_to_api(d[None], [2])[0]
    assert api.tolist() == [2, 3, 0, 1, -1]


def test_star_and_duplicates():
    g = Csr(4, [(0, 1), (0, 1), (0, 2), (2, 3), (3, 0)])
    assert O.bfs_queue(g, 0)[0].tolist() == [0, 1, 1, 2]
    assert O.bfs_queue(g, 3)[0].tolist() == [1, 2, 2, 0]


def test_sssp_hand():
    # 0->1 (4), 0->2 (1), 2->1 (2), 1->3 (1)
    g = Csr(5, None, weights=[(0, 1, 4.0), (0, 2, 1.0), (2, 1, 2.0), (1, 3, 1.0)])
    d = O.sssp(g, 0)
    assert d.tolist()[:4] == [0.0, 3.0, 1.0, 4.0]
    assert d[4] == FLT_MAX


def test_sssp_last_duplicate_of_source_row_wins():
    # Reference quirk (src/algorithm/cpu/sssp.cpp:41-45): the source row seeds
    # its neighbours in CSR order, so the later duplicate (5) survives.
    g = Csr(3, None, weights=[(0, 1, 3.0), (0, 1, 5.0), (1, 2, 1.0)])
    assert O.sssp(g, 0).tolist() == [0.0, 5.0, 6.0]


def test_closeness_formulas():
    d = np.array([0, 1, 2, 0, 1], np.int32)  # source 0, vertex 3 unreachable
    assert O.closeness_hops(d, 0) == pytest.approx(4 / 4)
    assert O.closeness_ref_int(d, 0) == 1.0
    dw = np.array([0, 2.5, FLT_MAX, 1.5], np.float32)
    assert O.closeness_weighted(dw, 0) == pytest.approx(3 / 4.0)


def test_golden_bfs(goldens):
    for g in goldens:
        for i, s in enumerate(g.sources):
            d, _ = O.bfs_queue(g, s)
            assert np.array_equal(d, g.bfs_ref[i]), (g.name, s)
            assert np.array_equal(O.bfs_bitmap(g, s), g.bfs_ref[i]), (g.name, s)


def test_golden_sssp(goldens):
    for g in goldens:
        if g.sssp_ref is None:
            continue
        for i, s in enumerate(g.sources):
            d = O.sssp(g, s)
            ref = g.sssp_ref[i].copy()
            # the reference's text output omits 0-valued entries (the source)
            d0 = d.copy()
            d0[d0 == 0] = 0
            assert np.array_equal(d0, ref), (g.name, s)


def test_golden_closeness_text(goldens):
    for g in goldens:
        for i, s in enumerate(g.sources):
            d, _ = O.bfs_queue(g, s)
            assert "Closeness Centrality:%3.5f" % O.closeness_ref_int(d, s) == g.cc_text[i]


def test_golden_mssp(goldens):
    for g in goldens:
        if g.mssp_ref is None:
            continue
        d, _, skipped = O.mssp(g, g.mssp_sources)
        assert np.array_equal(d, g.mssp_ref), g.name
        assert not skipped.any()


@pytest.mark.skipif(not O.ref_available(), reason="reference not compiled here")
@pytest.mark.parametrize("kind", ["er", "rmat", "grid", "knn"])
def test_port_matches_reference(kind):
    g = {"er": lambda: gen.erdos_renyi(2000, 16000, seed=5, weights=True),
         "rmat": lambda: gen.rmat(11, 8, seed=6, weights=True),
         "grid": lambda: gen.grid(40, 37, weights=True),
         "knn": lambda: gen.knn(3000, 5, seed=7, weights=True)}[kind]()
    srcs = gen.sources(g, 6, seed=9)
    for s in srcs:
        assert np.array_equal(O.bfs_queue(g, s)[0], O.ref_bfs_kernel(g, s))
        assert np.array_equal(O.bfs_bitmap(g, s), O.ref_bfs_bitmap(g, s))
        assert np.array_equal(O.sssp(g, s), O.ref_sssp(g, s))
        d, _ = O.bfs_queue(g, s)
        assert O.closeness_ref_int(d, s) == O.ref_cc(g, s)
    d, e, _ = O.mssp(g, srcs)
    dr, _ = O.ref_mssp(g, srcs)
    assert np.array_equal(d, dr)


@pytest.mark.skipif(not O.ref_available(), reason="reference not compiled here")
def test_port_matches_reference_with_duplicates_and_self_loops():
    rng = np.random.default_rng(3)
    n = 400
    src = rng.integers(0, n, 3000)
    dst = rng.integers(0, n, 3000)
    dst[:200] = src[:200]  # self loops
    w = rng.integers(1, 10, 3000).astype(np.float32)
    order = np.lexsort((w, dst, src))
    g = Csr(n, [(int(a), int(b)) for a, b in zip(src[order], dst[order])])
    g.w_f32 = w[order]
    g.col = dst[order].astype(np.int32)
    for s in range(0, n, 37):
        assert np.array_equal(O.bfs_queue(g, s)[0], O.ref_bfs_kernel(g, s))
        assert np.array_equal(O.sssp(g, s), O.ref_sssp(g, s))


def test_bc_hand_path():
    # path 0-1-2 (both directions): sources 0 and 2 each credit vertex 1
    # with 1 (its successor has one predecessor); source 1 credits nobody
    g = Csr(3, [(0, 1), (1, 0), (1, 2), (2, 1)])
    assert np.allclose(O.bc(g), [0.0, 2.0, 0.0])
    assert O.bc(g, [0]).tolist() == [0.0, 1.0, 0.0]


def test_bc_hand_diamond():
    # 0 -> {1, 2} -> 3 -> 4 (directed): from 0, vertex 3 has two
    # predecessors (1/2 each) and passes its own 1 (from 4) on undivided
    g = Csr(5, [(0, 1), (0, 2), (1, 3), (2, 3), (3, 4)])
    d = O.bc(g, [0])
    assert np.allclose(d, [0.0, 1.5, 1.5, 1.0, 0.0])


@pytest.mark.skipif(not O.ref_available(), reason="reference not built here")
def test_bc_port_matches_reference():
    # the float32 restatement repeats the reference's bc_cpu bit for bit; the
    # float64 one agrees to float32 rounding
    graphs = [gen.rmat(8, 8, seed=81), gen.erdos_renyi(300, 1500, seed=82), gen.grid(9, 13),
              gen.rmat(7, 4, seed=83)]
    # duplicates and a self loop, as a hand-filled CSR may carry
    rp = np.array([0, 3, 5, 7, 8], np.int32)
    col = np.array([1, 1, 2, 0, 3, 3, 2, 3], np.int32)
    graphs.append(gen.CsrGraph(4, rp, col))
    for g in graphs:
        want = O.ref_bc(g)
        got = O.bc(g, exact_ref_order=True)
        assert np.array_equal(got, want), g.n
        d = O.bc(g)
        np.testing.assert_allclose(d, want.astype(np.float64), rtol=1e-5, atol=1e-4)
