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
