"""Autotuner and the speed options it sets: the settings change speed only
(distances stay the oracle's), the cache hands a graph class's settings to
a new handle, and the cache file round-trips."""

import numpy as np
import pytest

import oracle as O
from dawn_gb300 import abi, gen

pytestmark = pytest.mark.gpu


def expected(g, srcs):
    ref, edges, _ = O.mssp(g, srcs)
    return O.hops_ref_to_api(ref, srcs), edges


@pytest.mark.parametrize("seg,bps", [(128, 1), (8192, 2), (1024, 0)])
def test_pull_segment_and_grid_size_change_nothing(seg, bps):
    g = gen.rmat(17, 32, a=0.62, b=0.17, c=0.17, seed=14)  # rows with tens of thousands of in-edges
    srcs = gen.sources(g, 100, seed=15)
    want, edges = expected(g, srcs)
    with abi.Graph(g) as dg:
        d0, _ = dg.bfs(srcs, variant=abi.VARIANT_BITSET)  # graphs captured with the defaults
        dg.set_option(abi.OPT_PULL_SEGMENT, seg)
        dg.set_option(abi.OPT_BLOCKS_PER_SM, bps)
        assert dg.get_option(abi.OPT_PULL_SEGMENT) == seg and dg.get_option(abi.OPT_BLOCKS_PER_SM) == bps
        for v in (abi.VARIANT_BITSET, abi.VARIANT_LEARNED, abi.VARIANT_DO):
            k = 100 if v != abi.VARIANT_DO else 3
            d, st = dg.bfs(srcs[:k], variant=v)
            assert np.array_equal(d, want[:k]), (seg, bps, v)
        assert np.array_equal(d0, want)


def test_autotune_and_cache(tmp_path):
    g = gen.rmat(15, 16, seed=51)
    srcs = gen.sources(g, 200, seed=52)
    want, _ = expected(g, srcs)
    with abi.Graph(g) as dg:
        t = dg.autotune(srcs)
        assert t["from_cache"] == 0 and t["ms"] > 0 and t["default_ms"] > 0
        assert t["ms"] <= t["default_ms"] * 1.0001
        assert t["bitset_width"] in (1, 2, 4) and t["push_ratio"] in (2, 4, 8, 16)
        assert dg.get_option(abi.OPT_PUSH_RATIO) == t["push_ratio"]
        assert dg.get_option(abi.OPT_AUTO_LEARNED) == t["learned"]
        d, _ = dg.bfs(srcs)
        assert np.array_equal(d, want)
    # a second graph of the same class takes the cached settings
    g2 = gen.rmat(15, 16, seed=53)
    s2 = gen.sources(g2, 200, seed=54)
    with abi.Graph(g2) as dg2:
        t2 = dg2.autotune(s2, use_cache=True)
        assert t2["from_cache"] == 1
        for k in ("bitset_width", "push_ratio", "pull_segment", "blocks_per_sm", "learned"):
            assert t2[k] == t[k]
        w2, _ = expected(g2, s2)
        d2, _ = dg2.bfs(s2)
        assert np.array_equal(d2, w2)
    path = tmp_path / "tune.txt"
    abi.tune_cache_save(str(path))
    text = path.read_text()
    assert "|n15|" in text
    abi.tune_cache_load(str(path))


def test_autotune_single_source():
    g = gen.rmat(14, 8, seed=55)
    srcs = gen.sources(g, 1, seed=56)
    want, _ = expected(g, srcs)
    with abi.Graph(g) as dg:
        t = dg.autotune(srcs)
        assert t["bitset_width"] == 0 and t["blocks_per_sm"] in (0, 1, 2, 4)
        d, _ = dg.bfs(srcs, variant=abi.VARIANT_DO)
        assert np.array_equal(d, want)


def test_l2_window_changes_nothing():
    g = gen.rmat(14, 16, seed=57)
    srcs = gen.sources(g, 64, seed=58)
    want, _ = expected(g, srcs)
    with abi.Graph(g) as dg:
        assert dg.get_option(abi.OPT_L2_PERSIST) == 0
        for persist in (1, 0, 1):
            dg.set_option(abi.OPT_L2_PERSIST, persist)
            d, _ = dg.bfs(srcs, variant=abi.VARIANT_LEARNED)
            assert np.array_equal(d, want), persist
