"""Closeness centrality against the oracle's float64 restatement (1e-6 relative)."""

import numpy as np
import pytest

import oracle as O
from dawn_gb300 import abi, gen

pytestmark = pytest.mark.gpu
RTOL = 1e-6


def test_hops_closeness():
    g = gen.rmat(13, 16, seed=21)
    srcs = gen.sources(g, 100, seed=22)
    ref, _, _ = O.mssp(g, srcs)
    want = np.array([O.closeness_hops(ref[i], s) for i, s in enumerate(srcs)])
    with abi.Graph(g) as dg:
        cc, sums, reached = dg.closeness(srcs)
    np.testing.assert_allclose(cc, want, rtol=RTOL, atol=0)
    api = O.hops_ref_to_api(ref, srcs)
    assert np.array_equal(reached, (api > 0).sum(axis=1))
    # the reference's literal integer-division value is recoverable
    lit = np.array([O.closeness_ref_int(ref[i], s) for i, s in enumerate(srcs)])
    assert np.array_equal(np.floor((g.n - 1) / sums).astype(np.float32), lit)


@pytest.mark.parametrize("w", ["i32", "f32"])
def test_weighted_closeness(w):
    g = gen.rmat(12, 8, seed=23, weights=True)
    srcs = gen.sources(g, 12, seed=24)
    ref = O.msssp(g, srcs)
    want = np.array([O.closeness_weighted(ref[i], s) for i, s in enumerate(srcs)])
    with abi.Graph(g, weights=w) as dg:
        cc, _, _ = dg.closeness(srcs, weighted=True)
    np.testing.assert_allclose(cc, want, rtol=RTOL, atol=0)


@pytest.mark.parametrize("width", [1, 2, 4])
def test_all_vertex_closeness(width):
    # every vertex a source (the all-pairs closeness), at each batch width;
    # directed graph with unreachable pairs, duplicates in the source list
    g = gen.erdos_renyi(3000, 9000, seed=25)
    srcs = np.concatenate([np.arange(g.n, dtype=np.int32), np.array([0, 0, 17], np.int32)])
    ref, _, _ = O.mssp(g, srcs)
    want = np.array([O.closeness_hops(ref[i], s) for i, s in enumerate(srcs)])
    api = O.hops_ref_to_api(ref, srcs)
    with abi.Graph(g) as dg:
        dg.set_option(abi.OPT_BITSET_WIDTH, width)
        cc, sums, reached = dg.closeness(srcs)
    np.testing.assert_allclose(cc, want, rtol=RTOL, atol=0)
    assert np.array_equal(reached, (api > 0).sum(axis=1))
    assert np.array_equal(sums, np.where(api > 0, api, 0).sum(axis=1).astype(np.float64))


def test_closeness_high_diameter():
    # levels past 2^8: the distance sums use every level slice
    g = gen.grid(3, 700)
    srcs = np.array([0, 1, 2099, 1050, 1050], np.int32)
    ref, _, _ = O.mssp(g, srcs)
    want = np.array([O.closeness_hops(ref[i], s) for i, s in enumerate(srcs)])
    with abi.Graph(g) as dg:
        cc, _, _ = dg.closeness(srcs)
    np.testing.assert_allclose(cc, want, rtol=RTOL, atol=0)


@pytest.mark.parametrize("width", [1, 4])
def test_closeness_deep_levels_many_sources(width):
    # every vertex of a grid a source: most pairs are reached past level 32,
    # where the sums are added level by level during the traversal
    g = gen.grid(12, 40)
    srcs = np.arange(g.n, dtype=np.int32)
    ref, _, _ = O.mssp(g, srcs)
    want = np.array([O.closeness_hops(ref[i], s) for i, s in enumerate(srcs)])
    api = O.hops_ref_to_api(ref, srcs)
    with abi.Graph(g) as dg:
        dg.set_option(abi.OPT_BITSET_WIDTH, width)
        cc, sums, reached = dg.closeness(srcs)
    np.testing.assert_allclose(cc, want, rtol=RTOL, atol=0)
    assert np.array_equal(reached, (api > 0).sum(axis=1))
    assert np.array_equal(sums, np.where(api > 0, api, 0).sum(axis=1).astype(np.float64))
