"""Invalid input is rejected on the host or by the upload-time validation
pass, with a status code and a message; nothing faults the device."""

import numpy as np
import pytest

from dawn_gb300 import abi, gen

pytestmark = pytest.mark.gpu


def bad(g, status=abi.ERR_INVALID_ARG, **kw):
    with pytest.raises(abi.DawnError) as e:
        abi.Graph(g, **kw)
    assert e.value.status == status
    return str(e.value)


def test_invalid_csr_rejected():
    rp = np.array([0, 2, 3], np.int32)
    assert "col index" in bad(gen.CsrGraph(2, rp, np.array([1, 5, 0], np.int32)))
    assert "decreases" in bad(gen.CsrGraph(2, np.array([0, 3, 2], np.int32), np.array([1, 0, 1], np.int32)))
    assert "row_ptr[n] != m" in bad(gen.CsrGraph(2, np.array([0, 1, 1], np.int32), np.array([1, 0], np.int32)))
    w = np.array([1, -2, 3], np.int32)
    assert "weight" in bad(gen.CsrGraph(2, rp, np.array([1, 0, 1], np.int32), w, w.astype(np.float32)),
                           weights="i32")
    wf = np.array([1, np.nan, 3], np.float32)
    assert "weight" in bad(gen.CsrGraph(2, rp, np.array([1, 0, 1], np.int32), w, wf), weights="f32")


def test_bad_sources_rejected():
    g = gen.rmat(8, 4, seed=1)
    with abi.Graph(g) as dg:
        for srcs in ([g.n], [-1], [0, 3, g.n + 7]):
            with pytest.raises(abi.DawnError) as e:
                dg.bfs(srcs)
            assert e.value.status == abi.ERR_INVALID_ARG
        d, st = dg.bfs([])
        assert d.shape == (0, g.n) and st.edges_traversed == 0
        with pytest.raises(abi.DawnError):
            dg.bfs([0], variant=99)
        # the handle stays usable after rejected calls
        d, _ = dg.bfs([0])
        assert d[0, 0] == 0


def test_bad_options_rejected():
    g = gen.rmat(8, 4, seed=2)
    with abi.Graph(g) as dg:
        for opt, val in ((abi.OPT_BITSET_WIDTH, 3), (abi.OPT_BITSET_WIDTH, 8), (abi.OPT_PUSH_RATIO, 0),
                         (99, 1)):
            with pytest.raises(abi.DawnError) as e:
                dg.set_option(opt, val)
            assert e.value.status == abi.ERR_INVALID_ARG
        assert dg.get_option(abi.OPT_BITSET_WIDTH) == 0
        assert dg.get_option(abi.OPT_PUSH_RATIO) == 4


def test_bad_selector_rejected():
    g = gen.rmat(8, 4, seed=3)
    with abi.Graph(g) as dg:
        with pytest.raises(abi.DawnError) as e:
            dg.set_selector(np.zeros(100, np.float32))
        assert e.value.status == abi.ERR_INVALID_ARG
        w = np.zeros(abi.SELECTOR_WEIGHTS, np.float32)
        w[7] = np.nan
        with pytest.raises(abi.DawnError):
            dg.set_selector(w)
        for bad in (-1, 4):
            with pytest.raises(abi.DawnError):
                dg.set_option(abi.OPT_FORCE_VARIANT, bad)
        dg.set_selector(None)
        d, _ = dg.bfs([0], variant=abi.VARIANT_LEARNED)
        assert d[0, 0] == 0
