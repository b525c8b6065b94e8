"""The C++ host layer (DAWN::Graph::createGraph and friends) against the
reference loader's CSR, recorded in the golden fixtures, and - where the
reference sources are present - the reference's own GPU command-line mains
compiled unchanged against this project's headers."""

import os
import subprocess

import numpy as np
import pytest

import oracle as O
from dawn_gb300 import BIN_DIR, HOST_DIR, INCLUDE_DIR, LIB_DIR, gen

REF = O.reference_dir() or ""


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


def test_csr_cache(goldens, tmp_path):
    # DAWN_CSR_CACHE: the first load parses and stores the CSR; an unchanged
    # file loads from the cache; a changed or damaged one is parsed again
    import shutil
    import time
    cache = tmp_path / "cache"
    cache.mkdir()
    env = dict(os.environ, DAWN_CSR_CACHE=str(cache))
    for g in goldens:
        mtx = tmp_path / os.path.basename(g.mtx)
        shutil.copy(g.mtx, mtx)

        def load():
            out = str(tmp_path / "csr.bin")
            r = subprocess.run([os.path.join(BIN_DIR, "dump_csr"), str(mtx), str(int(g.weighted)), "0", out],
                               stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, env=env)
            assert r.returncode == 0, r.stdout
            with open(out, "rb") as f:
                rows, _ = np.frombuffer(f.read(8), np.int32)
                nnz = int(np.frombuffer(f.read(8), np.int64)[0])
                f.read(8)
                rp = np.frombuffer(f.read(4 * (rows + 1)), np.int32)
                col = np.frombuffer(f.read(4 * nnz), np.int32)
                val = np.frombuffer(f.read(4 * nnz), np.float32) if g.weighted else None
            assert np.array_equal(rp, g.row_ptr) and np.array_equal(col, g.col), g.name
            if g.weighted:
                assert np.array_equal(val, g.w_f32), g.name
            files = list(cache.glob(mtx.name + ".*.dawncsr"))
            assert len(files) == 1, files
            return files[0], files[0].stat().st_mtime_ns

        path, t1 = load()
        assert (".d" if g.directed else ".s") in path.name
        _, t2 = load()
        assert t2 == t1  # read back, not rewritten
        st = mtx.stat()
        os.utime(mtx, ns=(st.st_atime_ns, st.st_mtime_ns + 1_000_000_000))
        time.sleep(0.01)
        _, t3 = load()
        assert t3 != t2  # the changed file was parsed again
        with open(path, "r+b") as f:
            f.truncate(40)
        _, t4 = load()
        assert t4 != t3 and path.stat().st_size > 40
        # damaged contents under an intact header: a column outside [0, n),
        # then a row pointer that decreases; each is parsed again (load()
        # checks the CSR equals the fixture's) and the cache rewritten
        header, t = 48, t4
        if g.m == 0:
            continue
        for offset, value in ((header + 4 * (g.n + 1), g.n), (header + 4, g.row_ptr[1] + g.m + 1)):
            with open(path, "r+b") as f:
                f.seek(offset)
                f.write(np.array([value], np.int32).tobytes())
            time.sleep(0.01)
            _, t_new = load()
            assert t_new != t, (g.name, offset)
            t = t_new


def test_outfile_text_matches_printf(tmp_path):
    # the parallel writer produces the bytes of the printf formats the
    # reference's ostream output amounts to (%d, %g, %.6f)
    exe = str(tmp_path / "outfile_check")
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cpp", "outfile_check.cpp")
    r = subprocess.run(["g++", "-std=c++17", src, "-I", os.path.join(HOST_DIR, "include"), "-I", INCLUDE_DIR,
                        "-fopenmp", "-o", exe, "-L", LIB_DIR, "-ldawn_host", "-ldawn_gb300",
                        "-Wl,-rpath," + LIB_DIR], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    rng = np.random.default_rng(3)
    n, source = 200_000, 777
    iv = rng.integers(-5, 1 << 20, n).astype(np.int32)
    iv[:6] = [0, -1, 2**31 - 1, -2**31, 1, 10**9]
    fv = (rng.standard_normal(n) * 10.0 ** rng.integers(-8, 9, n)).astype(np.float32)
    fv[:7] = [0.0, np.float32(3.4028235e38), np.float32(1e-40), -0.0, 1.0, np.float32(123456.78), np.nan]
    fv[rng.integers(0, n, 5000)] = 0.0
    inp = tmp_path / "vals.bin"
    with open(inp, "wb") as f:
        f.write(np.array([n, source], np.int32).tobytes() + iv.tobytes() + fv.tobytes())
    r = subprocess.run([exe, str(inp), str(tmp_path / "out")], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True)
    assert r.returncode == 0, r.stdout
    want_is = "".join("%d %d %d\n" % (source, j, v) for j, v in enumerate(iv.tolist()) if j != source and v > 0)
    want_fs = "".join("%d %d %g\n" % (source, j, v) for j, v in enumerate(fv.tolist()) if j != source and v != 0)
    want_i = "".join("%d %d\n" % (j, v) for j, v in enumerate(iv.tolist()) if v > 0)
    want_f = "".join("%d %.6f\n" % (j, v) for j, v in enumerate(fv.tolist()) if v != 0)
    for ext, want in ((".is", want_is), (".fs", want_fs), (".i", want_i), (".f", want_f)):
        got = (tmp_path / ("out" + ext)).read_text()
        assert got == want, ext


def test_dedup_option(goldens, tmp_path):
    # DAWN_DEDUP=1 (opt-in, not in the reference): an unweighted read drops
    # repeated (row, col) entries; a weighted read keeps them
    env = dict(os.environ, DAWN_DEDUP="1")
    for g in goldens:
        out = str(tmp_path / "csr.bin")
        r = subprocess.run([os.path.join(BIN_DIR, "dump_csr"), g.mtx, str(int(g.weighted)), "0", out],
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, env=env)
        assert r.returncode == 0, r.stdout
        with open(out, "rb") as f:
            rows, _ = np.frombuffer(f.read(8), np.int32)
            nnz = int(np.frombuffer(f.read(8), np.int64)[0])
            f.read(8)
            rp = np.frombuffer(f.read(4 * (rows + 1)), np.int32)
            col = np.frombuffer(f.read(4 * nnz), np.int32)
        if g.weighted:
            assert np.array_equal(rp, g.row_ptr) and np.array_equal(col, g.col), g.name
            continue
        # the golden CSR (duplicates kept, rows sorted) with repeats removed
        deg = np.diff(g.row_ptr.astype(np.int64))
        row = np.repeat(np.arange(g.n), deg)
        keep = np.ones(len(g.col), bool)
        keep[1:] = (row[1:] != row[:-1]) | (g.col[1:] != g.col[:-1])
        want_rp = np.concatenate([[0], np.cumsum(np.bincount(row[keep], minlength=g.n))])
        assert np.array_equal(rp, want_rp), g.name
        assert np.array_equal(col, g.col[keep]), g.name
        if g.name.startswith("dups"):
            assert keep.sum() < len(g.col), g.name  # the fixture does hold repeats
