"""CPU checks of the drop-in boundary: the library loads and exports every
entry point include/dawn_gb300.h declares (no compute call without a GPU),
and the generators are deterministic."""

import hashlib
import os
import re

import numpy as np

from dawn_gb300 import INCLUDE_DIR, abi, gen


def declared_symbols():
    text = open(os.path.join(INCLUDE_DIR, "dawn_gb300.h")).read()
    return sorted(set(re.findall(r"^(?:dawn_status|const char\*)\s+(dawn_\w+)\(", text, re.M)))


def test_header_declares_what_bindings_expect():
    assert declared_symbols() == sorted(abi.EXPORTS)


def test_library_exports_every_declared_symbol():
    L = abi.lib()
    for name in declared_symbols():
        assert hasattr(L, name), name
    assert abi.version().startswith("dawn_gb300")
    assert L.dawn_last_error() == b""


def test_generators_deterministic():
    a = gen.rmat(10, 8, seed=123, weights=True)
    b = gen.rmat(10, 8, seed=123, weights=True)
    assert np.array_equal(a.row_ptr, b.row_ptr) and np.array_equal(a.col, b.col)
    assert np.array_equal(a.w_i32, b.w_i32)
    # rows sorted, unique, no self loops, symmetric
    for u in range(a.n):
        r = a.col[a.row_ptr[u]:a.row_ptr[u + 1]]
        assert np.all(np.diff(r) > 0) and not np.any(r == u)
    pairs = set(zip(np.repeat(np.arange(a.n), np.diff(a.row_ptr)).tolist(), a.col.tolist()))
    assert all((v, u) in pairs for u, v in pairs)
    # weights symmetric and in [1, 63]
    assert a.w_i32.min() >= 1 and a.w_i32.max() <= 63
    assert np.array_equal(a.w_f32, a.w_i32.astype(np.float32))
    # fixed digest: the same graph on every machine and thread count
    h = hashlib.sha256(a.row_ptr.tobytes() + a.col.tobytes() + a.w_i32.tobytes()).hexdigest()
    assert h == RMAT10_DIGEST, h


def test_er_and_grid_shapes():
    g = gen.erdos_renyi(65536, 1 << 20, seed=1)
    assert g.n == 65536 and 1_040_000 < g.m <= 1 << 20
    gr = gen.grid(4, 5)
    assert gr.m == 2 * (4 * 4 + 3 * 5)
    k = gen.knn(1000, 8, seed=2)
    assert k.degrees().min() >= 8


def test_sources_in_largest_component():
    g = gen.rmat(12, 4, seed=3)
    s = gen.sources(g, 64, seed=4)
    assert len(set(s.tolist())) == 64
    assert np.all(g.degrees()[s] > 0)


RMAT10_DIGEST = "49028ba9ecab84aa05bc4b8b11571e4c647ea492bcf13cf3f8c59762f05e7a40"


def test_tune_cache_file_checks(tmp_path):
    # host-only: the cache file is parsed and validated without a GPU
    good = tmp_path / "good.txt"
    good.write_text("# comment\nGB300|n22|d5|sym|s2 1 4 1024 0 1 2.2 2.25\n")
    abi.tune_cache_load(str(good))
    for bad in ("GB300|n22|d5|sym|s2 3 4 1024 0 1 2.2 2.25\n", "x 1 4\n", "k 1 0 1024 0 0 1 1\n"):
        p = tmp_path / "bad.txt"
        p.write_text(bad)
        try:
            abi.tune_cache_load(str(p))
        except abi.DawnError as e:
            assert e.status == abi.ERR_INVALID_ARG
        else:
            raise AssertionError("malformed cache accepted: " + bad)
    out = tmp_path / "out.txt"
    abi.tune_cache_save(str(out))
    assert "GB300|n22|d5|sym|s2 1 4 1024 0 1" in out.read_text()
