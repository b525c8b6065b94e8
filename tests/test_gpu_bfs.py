"""Hop distances through the C ABI against the oracle (bit-exact)."""

import numpy as np
import pytest

import oracle as O
from dawn_gb300 import abi, gen

pytestmark = pytest.mark.gpu

VARIANTS = [abi.VARIANT_PUSH, abi.VARIANT_DO, abi.VARIANT_BITSET, abi.VARIANT_AUTO]


def expected(g, srcs):
    ref, edges, _ = O.mssp(g, srcs)
    return O.hops_ref_to_api(ref, srcs), edges


def check(g, srcs, variants=VARIANTS, symmetric=None):
    want, edges = expected(g, srcs)
    with abi.Graph(g, symmetric=symmetric) as dg:
        for v in variants:
            d, st = dg.bfs(srcs, variant=v)
            bad = np.argwhere(d != want)
            assert bad.size == 0, (v, bad[:5], d[tuple(bad[0])], want[tuple(bad[0])])
            assert st.edges_traversed == edges, (v, st.edges_traversed, edges)


def test_golden(goldens):
    for g in goldens:
        check(g, g.sources)
        want = O.hops_ref_to_api(g.bfs_ref, g.sources)
        with abi.Graph(g) as dg:
            d, _ = dg.bfs(g.sources)
            assert np.array_equal(d, want), g.name


def test_directed_er_64k():
    # The CPU-runnable workload: directed ER, n = 65,536, 2^20 edges drawn.
    g = gen.erdos_renyi(65536, 1 << 20, seed=1)
    check(g, gen.sources(g, 64, seed=2, from_lcc=False))


@pytest.mark.parametrize("nsrc", [1, 2, 63, 64, 65, 130])
def test_rmat_batch_boundaries(nsrc):
    g = gen.rmat(14, 16, seed=3)
    srcs = gen.sources(g, nsrc, seed=nsrc)
    check(g, srcs, variants=[abi.VARIANT_BITSET, abi.VARIANT_DO])


def test_duplicate_and_isolated_sources():
    g = gen.rmat(12, 4, seed=4)
    iso = np.nonzero(g.degrees() == 0)[0]
    assert len(iso) > 0
    s = gen.sources(g, 10, seed=5)
    srcs = np.concatenate([s[:5], s[:3], iso[:2], s[5:]]).astype(np.int32)
    check(g, srcs)


def test_high_diameter_grid():
    g = gen.grid(60, 170)
    check(g, np.array([0, 60 * 170 - 1, 5000], np.int32))


def test_knn():
    g = gen.knn(20000, 8, seed=6)
    check(g, gen.sources(g, 40, seed=7))


def test_unsorted_rows_self_loops_duplicates():
    rng = np.random.default_rng(8)
    n = 3000
    src = rng.integers(0, n, 40000)
    dst = rng.integers(0, n, 40000)
    dst[:500] = src[:500]
    order = np.argsort(src, kind="stable")  # rows grouped, columns unsorted
    g = gen.CsrGraph(n, np.concatenate([[0], np.cumsum(np.bincount(src, minlength=n))]).astype(np.int32),
                     dst[order].astype(np.int32))
    check(g, np.arange(0, n, 97, dtype=np.int32))


def test_single_vertex_and_edgeless():
    g1 = gen.CsrGraph(1, np.array([0, 0], np.int32), np.zeros(0, np.int32))
    with abi.Graph(g1) as dg:
        for v in VARIANTS:
            d, st = dg.bfs([0, 0], variant=v)
            assert d.tolist() == [[0], [0]] and st.edges_traversed == 0
    g2 = gen.CsrGraph(70, np.zeros(71, np.int32), np.zeros(0, np.int32))
    with abi.Graph(g2) as dg:
        d, _ = dg.bfs(np.arange(70, dtype=np.int32), variant=abi.VARIANT_BITSET)
        assert np.array_equal(d, np.where(np.eye(70, dtype=bool), 0, -1))


def test_repeated_calls_reuse_graph():
    g = gen.rmat(13, 8, seed=9)
    srcs = gen.sources(g, 100, seed=10)
    want, _ = expected(g, srcs)
    with abi.Graph(g) as dg:
        for _ in range(3):
            for v in (abi.VARIANT_BITSET, abi.VARIANT_DO):
                d, _ = dg.bfs(srcs, variant=v)
                assert np.array_equal(d, want)


def hub_graph(nhub=1500, deg=2100, nleaf=5000, seed=12):
    """A root joined to nhub hubs of ~deg leaves each: the second level is
    more long rows than one shared-memory tile holds."""
    rng = np.random.default_rng(seed)
    n = 1 + nhub + nleaf
    src = [np.zeros(nhub, np.int64)]
    dst = [1 + np.arange(nhub)]
    for h in range(nhub):
        leaves = 1 + nhub + rng.choice(nleaf, deg, replace=False)
        src.append(np.full(deg, 1 + h))
        dst.append(leaves)
    src = np.concatenate(src)
    dst = np.concatenate(dst)
    s2 = np.concatenate([src, dst])
    d2 = np.concatenate([dst, src])
    order = np.lexsort((d2, s2))
    rp = np.concatenate([[0], np.cumsum(np.bincount(s2, minlength=n))]).astype(np.int32)
    return gen.CsrGraph(n, rp, d2[order].astype(np.int32), symmetric=True)


def test_long_rows_span_tiles():
    g = hub_graph()
    check(g, np.array([0, 1, 1 + 1500 + 7], np.int32))
    check(g, np.arange(0, 200, dtype=np.int32), variants=[abi.VARIANT_BITSET])


def test_heavy_pull_rows():
    # hubs with in-degree in the tens of thousands: pull levels cut them into
    # segments combined across warps
    g = gen.rmat(17, 32, a=0.62, b=0.17, c=0.17, seed=14)
    assert g.degrees().max() > 20000
    srcs = gen.sources(g, 130, seed=15)
    check(g, srcs, variants=[abi.VARIANT_BITSET])


@pytest.mark.parametrize("width", [1, 2, 4])
def test_bitset_widths(width):
    # every batch width gives the same distances; 300 sources leave a ragged
    # last batch at each width
    g = gen.rmat(15, 16, seed=21)
    srcs = gen.sources(g, 300, seed=22)
    want, edges = expected(g, srcs)
    with abi.Graph(g) as dg:
        dg.set_option(abi.OPT_BITSET_WIDTH, width)
        assert dg.get_option(abi.OPT_BITSET_WIDTH) == width
        for ratio in (1, 4, 64):
            dg.set_option(abi.OPT_PUSH_RATIO, ratio)
            d, st = dg.bfs(srcs, variant=abi.VARIANT_BITSET)
            assert np.array_equal(d, want), (width, ratio)
            assert st.edges_traversed == edges
            assert st.batches == -(-len(srcs) // (64 * width))


def test_width_changes_on_one_handle():
    # a wider batch grows the handle's buffers; narrower widths run after it
    # must not use the buffers of before
    g = gen.rmat(14, 8, seed=23)
    srcs = gen.sources(g, 260, seed=24)
    want, _ = expected(g, srcs)
    with abi.Graph(g) as dg:
        for width, k in ((1, 40), (4, 260), (1, 40), (2, 130), (0, 260), (1, 64)):
            dg.set_option(abi.OPT_BITSET_WIDTH, width)
            d, _ = dg.bfs(srcs[:k], variant=abi.VARIANT_BITSET)
            assert np.array_equal(d, want[:k]), (width, k)


@pytest.mark.parametrize("force", [1, 2, 3])
def test_forced_variants_change_nothing(force):
    # every level forced to sparse push, bitmap pull or dense push (the
    # per-variant timings the selector is trained on) gives the same distances
    g = gen.rmat(14, 8, seed=41)
    srcs = gen.sources(g, 70, seed=42)
    want, edges = expected(g, srcs)
    with abi.Graph(g) as dg:
        dg.set_option(abi.OPT_FORCE_VARIANT, force)
        for v, k in ((abi.VARIANT_BITSET, 70), (abi.VARIANT_DO, 3), (abi.VARIANT_PUSH, 2)):
            d, st = dg.bfs(srcs[:k], variant=v)
            assert np.array_equal(d, want[:k]), (force, v)
            assert st.edges_traversed == (edges if k == 70 else st.edges_traversed)
        d, _ = dg.bfs(srcs[:40], variant=abi.VARIANT_BITSET)
        assert np.array_equal(d, want[:40])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_selector_changes_nothing(seed):
    # a selector with arbitrary weights makes arbitrary per-level choices;
    # the distances stay those of the oracle
    rng = np.random.default_rng(seed)
    w = (rng.standard_normal(abi.SELECTOR_WEIGHTS) * 0.5).astype(np.float32)
    g = gen.rmat(14, 8, seed=43)
    srcs = gen.sources(g, 130, seed=44)
    want, edges = expected(g, srcs)
    grid = gen.grid(40, 60)
    gs = np.array([0, 1234, 2399], np.int32)
    gwant, _ = expected(grid, gs)
    with abi.Graph(g) as dg, abi.Graph(grid) as dgrid:
        for h in (dg, dgrid):
            h.set_selector(w)
        for v in (abi.VARIANT_BITSET, abi.VARIANT_LEARNED, abi.VARIANT_DO):
            k = 130 if v != abi.VARIANT_DO else 4
            d, st = dg.bfs(srcs[:k], variant=v)
            assert np.array_equal(d, want[:k]), v
            d, _ = dgrid.bfs(gs, variant=v)
            assert np.array_equal(d, gwant), v
        dg.set_selector(None)
        d, _ = dg.bfs(srcs, variant=abi.VARIANT_BITSET)
        assert np.array_equal(d, want)


def directed_path(n):
    rp = np.arange(n + 1, dtype=np.int32)
    rp[-1] = n - 1
    return gen.CsrGraph(n, rp, np.arange(1, n, dtype=np.int32))


def test_small_levels_change_nothing():
    # single-source direction-optimising BFS with stretches of small levels
    # run inside one cluster launch, against the same calls with every level
    # its own launch: distances (against the oracle), edge counts and level
    # counts agree.  The path has more levels than one cluster launch runs;
    # RMAT frontiers grow past the small limits and shrink back; the hub
    # graph sends long rows through the segment lists inside the cluster.
    hub = gen.rmat(12, 4, seed=51)
    rp = np.concatenate([[0], np.cumsum(np.diff(hub.row_ptr) + np.where(np.arange(hub.n) == 7, 3000, 0))])
    col = []
    for v in range(hub.n):
        col.append(hub.col[hub.row_ptr[v]:hub.row_ptr[v + 1]])
        if v == 7:
            col.append(np.random.default_rng(52).integers(0, hub.n, 3000))
    hub = gen.CsrGraph(hub.n, rp.astype(np.int32), np.concatenate(col).astype(np.int32))
    cases = [(directed_path(1500), np.array([0, 700, 1499], np.int32)),
             (gen.grid(60, 170), np.array([0, 60 * 170 - 1, 5000], np.int32)),
             (gen.rmat(14, 8, seed=53), None),
             (hub, np.array([7, 8, 9], np.int32))]
    for g, srcs in cases:
        if srcs is None:
            srcs = gen.sources(g, 4, seed=54)
        want, edges = expected(g, srcs)
        with abi.Graph(g) as dg:
            assert dg.get_option(abi.OPT_SMALL_LEVELS) == 1
            on, st_on = dg.bfs(srcs, variant=abi.VARIANT_DO)
            dg.trace(True)
            traced, _ = dg.bfs(srcs, variant=abi.VARIANT_DO)
            dg.trace(False)
            dg.set_option(abi.OPT_SMALL_LEVELS, 0)
            off, st_off = dg.bfs(srcs, variant=abi.VARIANT_DO)
        for d in (on, traced, off):
            bad = np.argwhere(d != want)
            assert bad.size == 0, (g.n, bad[:5])
        assert st_on.edges_traversed == st_off.edges_traversed == edges
        assert st_on.levels == st_off.levels
        assert st_on.push_levels + st_on.pull_levels == st_off.push_levels + st_off.pull_levels


@pytest.mark.parametrize("width", [1, 2, 4])
def test_deep_levels_written_directly(width):
    # past level 32 the batched traversal writes new (source, vertex) pairs
    # out at once and the final pass keeps them: a grid (diameter 98) and a
    # directed path (levels up to 599) at every batch width, with ragged last
    # batches, duplicate sources and a source sitting at the far end; the
    # forced variants take the pull and dense paths past level 32 as well
    grid = gen.grid(40, 60)
    gsrc = np.concatenate([gen.sources(grid, 150, seed=61), [0, 0, grid.n - 1]]).astype(np.int32)
    path = directed_path(600)
    psrc = np.array([0, 1, 300, 599, 5], np.int32)
    for g, srcs in ((grid, gsrc), (path, psrc)):
        want, edges = expected(g, srcs)
        with abi.Graph(g) as dg:
            dg.set_option(abi.OPT_BITSET_WIDTH, width)
            for force in (0, 1, 2, 3):
                dg.set_option(abi.OPT_FORCE_VARIANT, force)
                d, st = dg.bfs(srcs, variant=abi.VARIANT_BITSET)
                bad = np.argwhere(d != want)
                assert bad.size == 0, (g.n, width, force, bad[:5])
                assert st.edges_traversed == edges


def broom(mids=40, leaves=100, seed=0):
    """Source 0 -> `mids` vertices -> `leaves` new leaves each -> one tail
    vertex per leaf, undirected.  The second level discovers mids x leaves
    vertices from rows shorter than 128 entries, more than one cluster CTA's
    frontier slice holds, so the cluster levels spill and hand back."""
    edges = []
    nxt = 1 + mids
    for i in range(mids):
        edges.append((0, 1 + i))
        for _ in range(leaves):
            edges.append((1 + i, nxt))
            nxt += 1
    first_leaf, last_leaf = 1 + mids, nxt
    for leaf in range(first_leaf, last_leaf):
        edges.append((leaf, nxt))
        nxt += 1
    e = np.array(edges, np.int64)
    e = np.concatenate([e, e[:, ::-1]])
    rng = np.random.default_rng(seed)
    w = rng.integers(1, 9, size=len(edges)).astype(np.int32)
    w = np.concatenate([w, w])
    order = np.lexsort((e[:, 1], e[:, 0]))
    e, w = e[order], w[order]
    rp = np.concatenate([[0], np.cumsum(np.bincount(e[:, 0], minlength=nxt))]).astype(np.int32)
    return gen.CsrGraph(nxt, rp, e[:, 1].astype(np.int32), w, w.astype(np.float32), symmetric=True)


def test_small_levels_slice_overflow():
    g = broom()
    srcs = np.array([0, 5], np.int32)
    want, edges = expected(g, srcs)
    with abi.Graph(g) as dg:
        on, st_on = dg.bfs(srcs, variant=abi.VARIANT_DO)
        dg.set_option(abi.OPT_SMALL_LEVELS, 0)
        off, st_off = dg.bfs(srcs, variant=abi.VARIANT_DO)
    assert np.array_equal(on, want) and np.array_equal(off, want)
    assert st_on.edges_traversed == st_off.edges_traversed == edges
