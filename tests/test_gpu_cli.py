"""The command-line tools end to end on a GPU: same flags, same output file
bytes and closeness line as the reference's tools (golden fixtures)."""

import os
import subprocess

import numpy as np
import pytest

from dawn_gb300 import BIN_DIR

pytestmark = pytest.mark.gpu


def run(tool, *args):
    r = subprocess.run([os.path.join(BIN_DIR, tool), *args], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True)
    assert r.returncode == 0, r.stdout
    return r.stdout


def test_bfs_output_bytes(goldens, tmp_path):
    for g in goldens:
        s = int(g.sources[0])
        out = str(tmp_path / (g.name + ".txt"))
        log = run("bfs_gpu", "-i", g.mtx, "-s", str(s), "-p", "true", "-o", out)
        assert open(out).read() == g.bfs_text0, g.name
        assert "Start print" in log and "Nodes:" in log


def test_sssp_output_bytes(goldens, tmp_path):
    for g in goldens:
        if g.sssp_text0 is None:
            continue
        s = int(g.sources[0])
        out = str(tmp_path / (g.name + ".w.txt"))
        run("sssp_gpu", "-i", g.mtx, "-s", str(s), "-p", "true", "-o", out)
        assert open(out).read() == g.sssp_text0, g.name


def test_cc_lines(goldens):
    for g in goldens:
        for i, s in enumerate(g.sources[:3]):
            log = run("cc_gpu", "-i", g.mtx, "-s", str(int(s)))
            line = [x for x in log.splitlines() if x.startswith("Closeness Centrality:")][0]
            assert line == g.cc_text[i], (g.name, s)
            if g.ccw_text is not None:
                log = run("cc_gpu", "-i", g.mtx, "-s", str(int(s)), "-w", "true")
                line = [x for x in log.splitlines() if x.startswith("Closeness Centrality:")][0]
                assert line == g.ccw_text[i], (g.name, s)


def test_mssp_apsp_print_the_graph_source(goldens, tmp_path):
    g = [x for x in goldens if x.name == "rmat_sym"][0]
    lst = str(tmp_path / "src.txt")
    with open(lst, "w") as f:
        f.write("\n".join(str(int(s)) for s in g.sources) + "\n")
    s0 = int(g.sources[0])
    out = str(tmp_path / "m.txt")
    log = run("mssp_gpu", "-i", g.mtx, "-l", lst, "-s", str(s0), "-p", "true", "-o", out)
    assert open(out).read() == g.bfs_text0
    assert "Time:" in log
    out2 = str(tmp_path / "a.txt")
    log = run("apsp_gpu", "-i", g.mtx, "-s", str(s0), "-p", "true", "-o", out2)
    assert open(out2).read() == g.bfs_text0
    assert "APSP start" in log and "APSP end" in log and "Progress: 100%" in log


def test_isolated_source_exits_zero(goldens):
    g = [x for x in goldens if x.name == "dups_general"][0]
    iso = int(np.nonzero(np.diff(g.row_ptr) == 0)[0][0])
    log = run("bfs_gpu", "-i", g.mtx, "-s", str(iso))
    assert f"Source [{iso}] is isolated node" in log


def test_bc_tool(goldens, tmp_path):
    # bc_gpu with the CPU tool's interface: "vertex value" lines (%.6f) for
    # the non-zero betweenness values of every vertex, all vertices sources
    import oracle as O
    for g in goldens:
        out = str(tmp_path / (g.name + ".bc.txt"))
        log = run("bc_gpu", "-i", g.mtx, "-o", out)
        assert "Nodes:" in log and "Edges:" in log and "Time:" in log
        got = np.zeros(g.n)
        for line in open(out):
            j, v = line.split()
            got[int(j)] = float(v)
        want = O.bc(g)
        np.testing.assert_allclose(got, want, rtol=1e-4, atol=2e-6 + 1e-6 * float(np.abs(want).max()))
