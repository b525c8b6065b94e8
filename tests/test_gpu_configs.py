"""Parity at the benchmark workloads themselves, not only at small shapes.

Every configuration the benchmark quotes is run here at its full size
through the C ABI and compared with the oracle, bit-exactly:

  - RMAT scale 22, edge factor 16, 64 sources (the headline step), batched
    (selector and heuristic, on the autotuned handle) and single-source;
  - the same topology with int32 and float32 weights in [1, 63], 64 sources
    batched and four single-source;
  - RMAT scale 18 with 4,096 sources, 256 per traversal (W = 4), every row;
  - 512 directed Erdos-Renyi graphs in one persistent launch, every part;
  - members of the mixed family: RMAT scale 24, the 2048 x 2048 grid and
    the 2^21-point kNN graph, a few sources each, every variant.

The contract is MSSP_CPU::run (src/algorithm/cpu/mssp.cpp:9-32) for hop
distances and SSSP_CPU::SSSP per source (src/algorithm/cpu/sssp.cpp:23-80)
for weighted ones.  Scale-only failure modes (int32 products of sources x n,
segment-list capacity at 1.3e8 edges, heavy pull rows of RMAT-22 hubs) only
show at these sizes.
"""

import os

import numpy as np
import pytest

import oracle as O
from dawn_gb300 import abi, gen

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
RMAT_A, RMAT_B, RMAT_C = 0.57, 0.19, 0.19


def first_mismatch(got, want):
    bad = np.argwhere(got != want)
    if bad.size == 0:
        return None
    i = tuple(bad[0])
    return (len(bad), i, got[i], want[i])


@pytest.fixture(scope="module")
def rmat22():
    # the benchmark's graph (seed 2022) and its 64 sources (seed 64); the
    # weighted generator draws the same topology as the unweighted one
    g = gen.rmat(22, 16, RMAT_A, RMAT_B, RMAT_C, seed=2022, weights=True)
    assert g.n == 1 << 22
    return g, gen.sources(g, 64, seed=64)


def test_rmat22_64_sources_headline(rmat22):
    g, srcs = rmat22
    ref, edges, _ = O.mssp(g, srcs, threads=THREADS)
    want = O.hops_ref_to_api(ref, srcs)
    del ref
    with abi.Graph(g) as dg:
        dg.autotune(srcs)  # the benchmark's handle settings
        for v in (abi.VARIANT_LEARNED, abi.VARIANT_BITSET, abi.VARIANT_AUTO):
            d, st = dg.bfs(srcs, variant=v)
            assert first_mismatch(d, want) is None, (v, first_mismatch(d, want))
            assert st.edges_traversed == edges, v
        d, st = dg.bfs(srcs[:4], variant=abi.VARIANT_DO)
        assert first_mismatch(d, want[:4]) is None, first_mismatch(d, want[:4])
        d, _ = dg.bfs(srcs[4:6], variant=abi.VARIANT_PUSH)
        assert first_mismatch(d, want[4:6]) is None


def to_ref(d):
    if d.dtype == np.float32:
        return d
    return np.where(d == abi.INT32_MAX, abi.FLT_MAX, d.astype(np.float32))


@pytest.mark.parametrize("w", ["i32", "f32"])
def test_rmat22_weighted_64_sources(rmat22, w):
    g, srcs = rmat22
    want = rmat22_weighted_oracle(g, srcs)
    reached = want != abi.FLT_MAX
    deg = g.degrees()
    with abi.Graph(g, weights=w) as dg:
        d, st = dg.sssp(srcs, variant=abi.VARIANT_AUTO)
        got = to_ref(d)
        assert first_mismatch(got, want) is None, (w, first_mismatch(got, want))
        assert st.edges_traversed == sum(int(deg[r].sum()) for r in reached)
        d, _ = dg.sssp(srcs[:4], variant=abi.VARIANT_DO)
        got = to_ref(d)
        assert first_mismatch(got, want[:4]) is None, (w, first_mismatch(got, want[:4]))


_weighted = {}


def rmat22_weighted_oracle(g, srcs):
    """SSSP_CPU::SSSP per source (each source on one thread, sources spread
    over the host's threads), computed once for both weight types: the
    float32 weights hold the same integer values as the int32 ones."""
    key = (g.n, g.m, tuple(int(s) for s in srcs))
    if key not in _weighted:
        _weighted.clear()
        _weighted[key] = O.msssp(g, srcs, threads=THREADS)
    return _weighted[key]


def test_rmat18_4096_sources_width4():
    g = gen.rmat(18, 16, RMAT_A, RMAT_B, RMAT_C, seed=2022)
    srcs = gen.sources(g, 4096, seed=64)
    with abi.Graph(g) as dg:
        dg.set_option(abi.OPT_BITSET_WIDTH, 4)
        for v in (abi.VARIANT_BITSET, abi.VARIANT_LEARNED):
            d, st = dg.bfs(srcs, variant=v)
            assert st.batches == 4096 // 256
            total = 0
            for i in range(0, 4096, 256):
                ref, edges, _ = O.mssp(g, srcs[i:i + 256], threads=THREADS)
                want = O.hops_ref_to_api(ref, srcs[i:i + 256])
                mm = first_mismatch(d[i:i + 256], want)
                assert mm is None, (v, i, mm)
                total += edges
            assert st.edges_traversed == total, v
            del d


def test_er512_family_one_launch():
    graphs, srcs = gen.er_family(ngraphs=512, seed=2022)
    u, off = gen.disjoint_union(graphs)
    with abi.Graph(u) as dg:
        dg.set_parts(off)
        blocks, st = dg.multi_bfs(srcs)
    total = 0
    for p, (g, s) in enumerate(zip(graphs, srcs)):
        ref, edges, _ = O.mssp(g, s, threads=THREADS)
        want = O.hops_ref_to_api(ref, s)
        mm = first_mismatch(blocks[p], want)
        assert mm is None, (p, g.n, mm)
        total += edges
    assert st.edges_traversed == total
    assert st.batches == sum(-(-len(s) // 64) for s in srcs)
    assert len(graphs) == 512 and sum(len(s) for s in srcs) > 512 * 8


def mixed_family_member(kind):
    """Held-out members of the selector's mixed family (same shapes and
    seeds as dawn_gb300.selector.family('heldout'))."""
    from dawn_gb300 import selector
    specs = {selector.spec_name(s): s for s in selector.family("heldout")}
    name = {"rmat24": "rmat24-a0.57", "grid": "grid2048", "knn": "knn2^21"}[kind]
    return selector.build(specs[name])


@pytest.mark.parametrize("kind,nsrc", [("rmat24", 4), ("knn", 6), ("grid", 6)])
def test_mixed_family_members(kind, nsrc):
    g = mixed_family_member(kind)
    srcs = gen.sources(g, nsrc, seed=99)
    ref, edges, _ = O.mssp(g, srcs, threads=THREADS)
    want = O.hops_ref_to_api(ref, srcs)
    del ref
    with abi.Graph(g) as dg:
        for v in (abi.VARIANT_LEARNED, abi.VARIANT_BITSET, abi.VARIANT_DO):
            d, st = dg.bfs(srcs, variant=v)
            assert first_mismatch(d, want) is None, (kind, v, first_mismatch(d, want))
            assert st.edges_traversed == edges, (kind, v)
