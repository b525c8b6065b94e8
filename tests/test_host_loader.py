"""The C++ host layer (DAWN::Graph::createGraph and friends) against the
reference loader's CSR, recorded in the golden fixtures, and - where the
reference sources are present - the reference's own GPU command-line mains
compiled unchanged against this project's headers."""

import os
import subprocess

import numpy as np
import pytest

from dawn_gb300 import BIN_DIR, HOST_DIR, INCLUDE_DIR, LIB_DIR, gen

REF = "/root/reference"


def dump(path, weighted, source, tmp):
    out = os.path.join(tmp, "csr.bin")
    r = subprocess.run([os.path.join(BIN_DIR, "dump_csr"), path, str(int(weighted)), str(source), out],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    with open(out, "rb") as f:
        rows, cols = np.frombuffer(f.read(8), np.int32)
        nnz = int(np.frombuffer(f.read(8), np.int64)[0])
        directed, src = np.frombuffer(f.read(8), np.int32)
        rp = np.frombuffer(f.read(4 * (rows + 1)), np.int32)
        col = np.frombuffer(f.read(4 * nnz), np.int32)
        val = np.frombuffer(f.read(4 * nnz), np.float32) if weighted else None
    return int(rows), rp, col, val, bool(directed), int(src), r.stdout


def test_loader_matches_reference_csr(goldens, tmp_path):
    for g in goldens:
        n, rp, col, val, directed, _, _ = dump(g.mtx, g.weighted, 0, str(tmp_path))
        assert n == g.n and directed == g.directed, g.name
        assert np.array_equal(rp, g.row_ptr), g.name
        assert np.array_equal(col, g.col), g.name
        if g.weighted:
            assert np.array_equal(val, g.w_f32), g.name


def test_loader_messages_and_source_modulo(goldens, tmp_path):
    g = [x for x in goldens if x.name == "rmat_sym_w"][0]
    *_, src, out = dump(g.mtx, False, 1000, str(tmp_path))
    assert src == 1000 % g.n
    assert "This is a weighted graph, and it has been instructed to use unweighted functions" in out
    assert "Read Input Graph" in out


def test_loader_large_parallel_parse(tmp_path):
    # big enough for the chunked parallel parser; compared with a numpy build
    g = gen.erdos_renyi(50000, 400000, seed=31)
    p = str(tmp_path / "big.mtx")
    gen.write_mtx(g, p)
    n, rp, col, _, directed, _, _ = dump(p, False, 0, str(tmp_path))
    assert directed and n == g.n
    assert np.array_equal(rp, g.row_ptr) and np.array_equal(col, g.col)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "algorithm", "gpu")), reason="reference sources absent")
@pytest.mark.parametrize("tool", ["bfs_gpu", "sssp_gpu", "mssp_gpu", "apsp_gpu", "cc_gpu"])
def test_reference_mains_build_against_this_api(tool, tmp_path):
    """The reference's own main() for each GPU tool, compiled unchanged
    against include/dawn/... of this project and linked with the host layer:
    the drop-in API check (no GPU needed to build)."""
    src = os.path.join(REF, "algorithm", "gpu", tool, tool + ".cu")
    exe = str(tmp_path / tool)
    r = subprocess.run(["g++", "-std=c++17", "-x", "c++", src, "-I", os.path.join(HOST_DIR, "include"),
                        "-I", INCLUDE_DIR, "-fopenmp", "-o", exe, "-L", LIB_DIR, "-ldawn_host", "-ldawn_gb300",
                        "-Wl,-rpath," + LIB_DIR], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
