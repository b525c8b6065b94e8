"""Many graphs in one call (dawn_graph_set_parts + dawn_multi_*): every
part's distance block equals the oracle's BFS of that part alone (bit-exact),
closeness agrees within 1e-6 relative, and malformed part layouts are
rejected."""

import numpy as np
import pytest

import oracle as O
from dawn_gb300 import abi, gen

pytestmark = pytest.mark.gpu


def check_parts(graphs, srcs):
    u, off = gen.disjoint_union(graphs)
    with abi.Graph(u) as dg:
        dg.set_parts(off)
        blocks, st = dg.multi_bfs(srcs)
        total_edges = 0
        for p, (g, s) in enumerate(zip(graphs, srcs)):
            if len(s) == 0:
                assert blocks[p].shape == (0, g.n)
                continue
            ref, edges, _ = O.mssp(g, s)
            want = O.hops_ref_to_api(ref, s)
            bad = np.argwhere(blocks[p] != want)
            assert bad.size == 0, (p, g.n, bad[:5])
            total_edges += edges
        assert st.edges_traversed == total_edges
        assert st.batches == sum(-(-len(s) // 64) for s in srcs)
        return dg, u, off


def grid_directed_path(rows, cols):
    g = gen.grid(rows, cols)
    return gen.CsrGraph(g.n, g.row_ptr, g.col, symmetric=True)


def test_mixed_parts_against_oracle():
    rng = np.random.default_rng(5)
    graphs, srcs = [], []
    # ER parts of assorted sizes and degrees
    for i in range(12):
        n = int(rng.integers(50, 4000))
        g = gen.erdos_renyi(n, int(n * rng.uniform(1, 20)), seed=100 + i)
        graphs.append(g)
        srcs.append(rng.integers(0, n, size=int(rng.integers(1, 64))).astype(np.int32))
    # a single vertex, an edgeless part, a part with no sources
    graphs.append(gen.CsrGraph(1, np.array([0, 0], np.int32), np.zeros(0, np.int32)))
    srcs.append(np.array([0, 0], np.int32))
    graphs.append(gen.CsrGraph(5, np.zeros(6, np.int32), np.zeros(0, np.int32)))
    srcs.append(np.array([4, 1], np.int32))
    graphs.append(gen.erdos_renyi(300, 900, seed=7))
    srcs.append(np.zeros(0, np.int32))
    # 130 sources in one part: three tasks; duplicates included
    g = gen.erdos_renyi(2000, 8000, seed=8)
    s = rng.integers(0, 2000, size=130).astype(np.int32)
    s[5] = s[6] = s[70]
    graphs.append(g)
    srcs.append(s)
    # high diameter: levels past 256 use slices beyond the register-held ones
    graphs.append(grid_directed_path(2, 400))
    srcs.append(np.array([0, 799, 400], np.int32))
    # RMAT part with hubs
    graphs.append(gen.rmat(12, 8, seed=9))
    srcs.append(gen.sources(graphs[-1], 64, seed=10))
    check_parts(graphs, srcs)


def test_er_family_shape():
    # the 512-graph workload's shape at a reduced count
    graphs, srcs = gen.er_family(ngraphs=48, seed=11)
    dg, u, off = check_parts(graphs, srcs)
    # repeated calls on one handle (the captured launch is replayed)
    with abi.Graph(u) as dg2:
        dg2.set_parts(off)
        a, _ = dg2.multi_bfs(srcs)
        b, _ = dg2.multi_bfs(srcs)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_multi_closeness():
    graphs, srcs = gen.er_family(ngraphs=10, nmin=500, nmax=5000, seed=12)
    u, off = gen.disjoint_union(graphs)
    with abi.Graph(u) as dg:
        dg.set_parts(off)
        cc, dsum, reached, _ = dg.multi_closeness(srcs)
    i = 0
    for g, s in zip(graphs, srcs):
        ref, _, _ = O.mssp(g, s)
        for k, src in enumerate(s):
            exp = O.closeness_hops(ref[k], src)
            assert abs(cc[i] - exp) <= 1e-6 * max(1.0, abs(exp)), (i, cc[i], exp)
            row = O.hops_ref_to_api(ref[k:k + 1], [src])[0]
            assert reached[i] == int(np.sum(row > 0))
            assert dsum[i] == float(np.sum(row[row > 0]))
            i += 1


def test_parts_rejected():
    a = gen.erdos_renyi(100, 400, seed=1)
    b = gen.erdos_renyi(50, 200, seed=2)
    u, off = gen.disjoint_union([a, b])
    with abi.Graph(u) as dg:
        # no parts declared yet
        so = np.array([0, 1, 2], np.int32)
        src = np.zeros(2, np.int32)
        out = np.empty(150, np.int32)
        rc = abi.lib().dawn_multi_bfs(dg.handle, so.ctypes.data, src.ctypes.data, out.ctypes.data, None)
        assert rc == abi.ERR_INVALID_ARG and b"set_parts" in abi.lib().dawn_last_error()
        for bad in ([0, 100], [0, 120, 150], [0, 100, 100, 150], [5, 100, 150]):
            with pytest.raises(abi.DawnError) as e:
                dg.set_parts(bad)
            assert e.value.status == abi.ERR_INVALID_ARG
        dg.set_parts(off)
        with pytest.raises(abi.DawnError):
            dg.multi_bfs([[100], [0]])
        with pytest.raises(abi.DawnError):
            dg.multi_bfs([[0], [-1]])
        blocks, _ = dg.multi_bfs([[0], [3]])
        assert blocks[0][0, 0] == 0 and blocks[1][0, 3] == 0
    # an edge that leaves its part
    col = u.col.copy()
    col[0] = 120
    bad = gen.CsrGraph(u.n, u.row_ptr, col)
    with abi.Graph(bad) as dg:
        with pytest.raises(abi.DawnError) as e:
            dg.set_parts(off)
        assert "leaves its part" in str(e.value)
    # a part above the per-part limit
    big = gen.CsrGraph(abi.PART_MAX_VERTICES + 1, np.zeros(abi.PART_MAX_VERTICES + 2, np.int32),
                       np.zeros(0, np.int32))
    with abi.Graph(big) as dg:
        with pytest.raises(abi.DawnError) as e:
            dg.set_parts([0, big.n])
        assert "limit" in str(e.value)
