"""Weighted distances (min-plus relax) through the C ABI against the oracle."""

import numpy as np
import pytest

import oracle as O
from dawn_gb300 import abi, gen

pytestmark = pytest.mark.gpu


def to_ref(d):
    """C-ABI int32 distances -> the reference's float encoding (FLT_MAX)."""
    if d.dtype == np.float32:
        return d
    return np.where(d == abi.INT32_MAX, abi.FLT_MAX, d.astype(np.float32))


def check(g, srcs, weights=("i32", "f32")):
    # AUTO runs the batched traversal (64 sources per pass) for two or more
    # sources, DO the single-source kernels; both must give the oracle's
    want = O.msssp(g, srcs)
    for w in weights:
        with abi.Graph(g, weights=w) as dg:
            for variant in (abi.VARIANT_AUTO, abi.VARIANT_DO):
                d, st = dg.sssp(srcs, variant=variant)
                got = to_ref(d)
                bad = np.argwhere(got != want)
                assert bad.size == 0, (w, variant, bad[:5])
                reached = want != abi.FLT_MAX
                assert st.edges_traversed == int((reached * g.degrees()[None, :]).sum()), variant


def test_golden(goldens):
    for g in goldens:
        if g.sssp_ref is None:
            continue
        check(g, g.sources)
        with abi.Graph(g, weights="f32") as dg:
            d, _ = dg.sssp(g.sources)
        d[d == 0] = 0
        assert np.array_equal(d, g.sssp_ref), g.name


def test_directed_er():
    g = gen.erdos_renyi(20000, 200000, seed=11, weights=True)
    check(g, gen.sources(g, 8, seed=12, from_lcc=False))


def test_rmat():
    g = gen.rmat(14, 16, seed=13, weights=True)
    check(g, gen.sources(g, 8, seed=14))


def test_grid_high_diameter():
    g = gen.grid(50, 90, seed=15, weights=True)
    check(g, np.array([0, 2222, 4499], np.int32))


def test_source_row_duplicates_last_wins():
    # 0->1 twice (3 then 5), 1->2 (1), 0->0 absent: the reference keeps 5.
    rp = np.array([0, 2, 3, 3], np.int32)
    col = np.array([1, 1, 2], np.int32)
    g = gen.CsrGraph(3, rp, col, np.array([3, 5, 1], np.int32), np.array([3, 5, 1], np.float32))
    want = O.msssp(g, [0])
    assert want.tolist() == [[0.0, 5.0, 6.0]]
    check(g, [0])
    check(g, [0, 0, 1])  # batched: every source bit resolves its row alone


def test_source_self_loop_is_expanded():
    # With a self loop the source enters the first frontier (alpha[source]),
    # so the shorter duplicate is found through it.
    rp = np.array([0, 3, 4, 4], np.int32)
    col = np.array([0, 1, 1, 2], np.int32)
    w = np.array([7, 3, 5, 1], np.int32)
    g = gen.CsrGraph(3, rp, col, w, w.astype(np.float32))
    want = O.msssp(g, [0])
    assert want.tolist() == [[0.0, 3.0, 4.0]]
    check(g, [0])
    check(g, [0, 2, 0])


def test_unweighted_graph_rejected():
    g = gen.rmat(8, 4, seed=1)
    with abi.Graph(g) as dg:
        with pytest.raises(abi.DawnError) as e:
            dg.sssp([0])
        assert e.value.status == abi.ERR_UNSUPPORTED


def test_long_rows_weighted():
    from test_gpu_bfs import hub_graph
    g = hub_graph(nhub=1200, deg=2100, nleaf=4000, seed=13)
    w = (np.arange(g.m) % 17 + 1).astype(np.int32)
    # symmetric weights are not needed for SSSP parity
    g.w_i32, g.w_f32 = w, w.astype(np.float32)
    check(g, np.array([0, 5, 1300], np.int32))


def asym_weights(g, seed):
    """Same topology, weights drawn per directed entry (so w(u,v) != w(v,u)):
    a pull level must read in-edge weights, not mirror the out-edges."""
    rng = np.random.default_rng(seed)
    wi = rng.integers(1, 64, g.m).astype(np.int32)
    return gen.CsrGraph(g.n, g.row_ptr, g.col, wi, wi.astype(np.float32), symmetric=g.symmetric)


@pytest.mark.parametrize("force", [1, 2, 0])
def test_forced_push_and_pull(force):
    # every level as push (1), every level as pull (2), or chosen per level
    # (0): the distances are the oracle's in each case
    graphs = [
        asym_weights(gen.rmat(14, 16, seed=61), 62),           # symmetric topology, asymmetric weights
        gen.erdos_renyi(20000, 200000, seed=63, weights=True),  # directed
        gen.rmat(16, 32, a=0.62, b=0.17, c=0.17, seed=64, weights=True),  # hubs: segmented pull rows
    ]
    for g in graphs:
        srcs = gen.sources(g, 5, seed=65, from_lcc=g.symmetric)
        want = O.msssp(g, srcs)
        for w in ("i32", "f32"):
            with abi.Graph(g, weights=w) as dg:
                dg.set_option(abi.OPT_FORCE_VARIANT, force)
                d, st = dg.sssp(srcs, variant=abi.VARIANT_DO)
                got = to_ref(d)
                bad = np.argwhere(got != want)
                assert bad.size == 0, (force, w, g.n, bad[:5])
                if force == 2:
                    assert st.pull_levels > 0
                if force == 1:
                    assert st.pull_levels == 0


@pytest.mark.parametrize("force,seg", [(1, 0), (2, 0), (2, 128), (0, 128)])
def test_batched_forced_push_and_pull(force, seg):
    # the batched traversal (AUTO, 70 sources: a full and a ragged batch) with
    # every level a push (1) or a pull (2), or chosen per level (0); a pull
    # segment of 128 in-edges makes every in-row of 256 or more a heavy row
    # cut into segment tasks, so the light and the heavy pull run side by
    # side.  In-degrees from 0 to over a thousand leave every count of live
    # tails per 32-entry batch and per lane group.
    graphs = [
        asym_weights(gen.rmat(14, 16, seed=61), 62),
        gen.erdos_renyi(20000, 200000, seed=63, weights=True),
        gen.rmat(16, 32, a=0.62, b=0.17, c=0.17, seed=64, weights=True),
    ]
    for g in graphs:
        srcs = gen.sources(g, 70, seed=85, from_lcc=g.symmetric)
        want = O.msssp(g, srcs)
        for w in ("i32", "f32"):
            with abi.Graph(g, weights=w) as dg:
                dg.set_option(abi.OPT_FORCE_VARIANT, force)
                if seg:
                    dg.set_option(abi.OPT_PULL_SEGMENT, seg)
                d, st = dg.sssp(srcs, variant=abi.VARIANT_AUTO)
                bad = np.argwhere(to_ref(d) != want)
                assert bad.size == 0, (force, seg, w, g.n, bad[:5])
                assert st.batches == 2
                if force == 2:
                    assert st.pull_levels > 0 and st.push_levels == 0
                if force == 1:
                    assert st.pull_levels == 0 and st.push_levels > 0


def test_pull_segment_sizes():
    g = gen.rmat(16, 32, a=0.62, b=0.17, c=0.17, seed=66, weights=True)
    srcs = gen.sources(g, 3, seed=67)
    want = O.msssp(g, srcs)
    with abi.Graph(g, weights="i32") as dg:
        dg.set_option(abi.OPT_FORCE_VARIANT, 2)
        for seg in (128, 1024, 8192):
            dg.set_option(abi.OPT_PULL_SEGMENT, seg)
            d, _ = dg.sssp(srcs, variant=abi.VARIANT_DO)
            assert np.array_equal(to_ref(d), want), seg


def test_batched_many_sources():
    # 150 sources: three batches (the last ragged), duplicates, isolated
    # sources and sources in other components
    g = gen.rmat(13, 8, seed=71, weights=True)
    iso = np.nonzero(g.degrees() == 0)[0]
    s = gen.sources(g, 140, seed=72)
    srcs = np.concatenate([s[:100], s[:5], iso[:3], s[100:]]).astype(np.int32)
    check(g, srcs)


def test_batched_directed_asymmetric():
    g = asym_weights(gen.erdos_renyi(5000, 60000, seed=73), 74)
    g = gen.CsrGraph(g.n, g.row_ptr, g.col, g.w_i32, g.w_f32, symmetric=False)
    check(g, gen.sources(g, 70, seed=75, from_lcc=False))


def test_batched_high_diameter_sparse_masks():
    # a weighted grid and a kNN graph, 100 sources: most frontier vertices
    # are active for a few sources at a time, so the relaxations run as
    # (vertex, source) pairs; a hub row mixes in the warp-per-vertex form
    g = gen.grid(40, 60, seed=76, weights=True)
    check(g, gen.sources(g, 100, seed=77))
    k = gen.knn(3000, 6, seed=78, weights=True)
    check(k, gen.sources(k, 70, seed=79))


def test_small_levels_change_nothing():
    # single-source weighted traversals whose small-frontier stretches run as
    # cluster levels, against the same calls with every level its own
    # launch and against the oracle: a weighted grid, a weighted path longer
    # than one cluster launch runs, a kNN graph and RMAT (hubs end the
    # cluster levels)
    n = 1300
    rp = np.arange(n + 1, dtype=np.int32)
    rp[-1] = n - 1
    w = (np.arange(n - 1) % 7 + 1).astype(np.int32)
    path = gen.CsrGraph(n, rp, np.arange(1, n, dtype=np.int32), w, w.astype(np.float32))
    cases = [(gen.grid(40, 60, seed=81, weights=True), 3), (path, 0), (gen.knn(3000, 6, seed=82, weights=True), 3),
             (gen.rmat(12, 8, seed=83, weights=True), 3)]
    for g, ns in cases:
        srcs = np.array([0, 1, 5], np.int32) if ns == 0 else gen.sources(g, ns, seed=84)
        want = O.msssp(g, srcs)
        for wt in ("i32", "f32"):
            with abi.Graph(g, weights=wt) as dg:
                assert dg.get_option(abi.OPT_SMALL_LEVELS) == 1
                on, st_on = dg.sssp(srcs, variant=abi.VARIANT_DO)
                dg.trace(True)
                traced, _ = dg.sssp(srcs, variant=abi.VARIANT_DO)
                dg.trace(False)
                dg.set_option(abi.OPT_SMALL_LEVELS, 0)
                off, st_off = dg.sssp(srcs, variant=abi.VARIANT_DO)
            for d in (on, traced, off):
                bad = np.argwhere(to_ref(d) != want)
                assert bad.size == 0, (g.n, wt, bad[:5])
            assert st_on.edges_traversed == st_off.edges_traversed


def test_small_levels_slice_overflow():
    # the broom of test_gpu_bfs: a cluster level finds more targets than a
    # CTA's slice holds
    from test_gpu_bfs import broom
    g = broom(seed=85)
    srcs = np.array([0, 5], np.int32)
    want = O.msssp(g, srcs)
    for wt in ("i32", "f32"):
        with abi.Graph(g, weights=wt) as dg:
            on, _ = dg.sssp(srcs, variant=abi.VARIANT_DO)
            dg.set_option(abi.OPT_SMALL_LEVELS, 0)
            off, _ = dg.sssp(srcs, variant=abi.VARIANT_DO)
        assert np.array_equal(to_ref(on), want) and np.array_equal(to_ref(off), want), wt
