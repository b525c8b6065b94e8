"""dawn_bfs_static, the entry point that allocates nothing (its working
memory is one static block of device memory per GPU), against the oracle's
MSSP_CPU::run and against dawn_bfs on a handle of the same CSR.  Distances
are integers, so the tolerance is zero.  Collected last so it also runs
after every other GPU test in one process."""

import numpy as np
import pytest

import oracle as O
from dawn_gb300 import abi, gen

pytestmark = pytest.mark.gpu


def _device(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _static(g, rp, col, source, dist, **kw):
    import torch
    abi.bfs_static(rp.data_ptr(), col.data_ptr(), g.n, g.m, int(source), dist.data_ptr(),
                   stream=torch.cuda.current_stream().cuda_stream, **kw)
    return dist.cpu().numpy()


@pytest.mark.parametrize("graph", ["rmat16", "er_directed_max_vertices"])
def test_static_matches_handle_path(graph):
    import torch
    if graph == "rmat16":
        g = gen.rmat(16, 8, seed=31)  # hubs: long rows travel as segments
    else:
        g = gen.erdos_renyi(abi.STATIC_MAX_VERTICES, 1 << 23, seed=33)
    srcs = gen.sources(g, 2, seed=32)
    ref, _, _ = O.mssp(g, srcs)
    want = O.hops_ref_to_api(ref, srcs)
    with abi.Graph(g) as dg:
        handle, _ = dg.bfs(srcs, variant=abi.VARIANT_PUSH)
    assert np.array_equal(handle, want)
    rp, col = _device(g.row_ptr), _device(g.col)
    dist = torch.empty(g.n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    # two calls in a row reuse the same scratch block
    for i, s in enumerate(srcs):
        got = _static(g, rp, col, s, dist)
        bad = np.argwhere(got != want[i])
        assert bad.size == 0, (graph, i, bad[:5])
    # and again, without the CSR check
    got = _static(g, rp, col, srcs[0], dist, flags=abi.GRAPH_NO_VALIDATE)
    assert np.array_equal(got, want[0])
    # a further call takes no device memory: the free figure does not move
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    got = _static(g, rp, col, srcs[1], dist)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert np.array_equal(got, want[1])


def test_static_rejects_what_it_cannot_hold():
    import torch
    g = gen.rmat(10, 4, seed=34)
    rp, col = _device(g.row_ptr), _device(g.col)
    dist = torch.empty(g.n, dtype=torch.int32, device="cuda")
    L = abi.lib()
    cases = [(abi.STATIC_MAX_VERTICES + 1, g.m, 0, "vertex limit"),
             (g.n, abi.STATIC_MAX_EDGES + 1, 0, "edge limit"),
             (g.n, g.m, g.n, "source")]
    for n, m, s, msg in cases:
        rc = L.dawn_bfs_static(rp.data_ptr(), col.data_ptr(), n, m, s, dist.data_ptr(), 0, None)
        assert rc == abi.ERR_INVALID_ARG and msg in L.dawn_last_error().decode(), (n, m, s)
    host = np.zeros(g.n, np.int32)
    rc = L.dawn_bfs_static(rp.data_ptr(), col.data_ptr(), g.n, g.m, 0, host.ctypes.data, 0, None)
    assert rc == abi.ERR_INVALID_ARG and b"current device" in L.dawn_last_error()
    # a column outside [0, n) is caught by the check before any traversal
    bad_col = _device(np.where(np.arange(g.m) == g.m // 2, g.n, g.col).astype(np.int32))
    torch.cuda.synchronize()
    rc = L.dawn_bfs_static(rp.data_ptr(), bad_col.data_ptr(), g.n, g.m, 0, dist.data_ptr(), 0, None)
    assert rc == abi.ERR_INVALID_ARG and b"col index" in L.dawn_last_error()
    # still usable afterwards
    with abi.Graph(g) as dg:
        want, _ = dg.bfs([0], variant=abi.VARIANT_PUSH)
    assert np.array_equal(_static(g, rp, col, 0, dist), want[0])
