"""Generates the golden fixtures under tests/golden/ by running the reference.

Run in a container that has the reference sources (default /root/reference):

    python tests/golden/make_golden.py [--ref /root/reference]

It compiles the reference's own command-line tools and loader from their
unmodified sources (oracle/Makefile, target `ref`), writes seeded small
graphs as MatrixMarket files, and records for each graph:
  * the CSR the reference loader builds (ref_dump_csr -> createGraph),
  * bfs_cpu / sssp_cpu / cc_cpu text output for a few sources (the tools'
    own `-p true -o file` output and stdout), weighted tools on one OpenMP
    thread (their relax races with more, see src/algorithm/cpu/sssp.cpp:186),
  * MSSP_CPU::run hop distances for a source list (in-process capture).
Everything lands in tests/golden/<name>.npz plus the .mtx inputs; the tests
read only those files, so they run where the reference is absent.
"""

import argparse
import os
import shutil
import subprocess
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "gal-dawn_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

FLT_MAX = np.float32(3.4028235e38)


def hand_written_inputs():
    """Loader edge cases the generators never produce (comments, duplicates,
    self loops, repeated weighted edges)."""
    files = {}
    files["dups_general"] = (
        "%%MatrixMarket matrix coordinate pattern general\n"
        "% a comment line\n"
        "7 7 12\n"
        "1 2\n1 2\n2 3\n3 3\n3 4\n4 1\n5 6\n6 5\n2 4\n4 2\n7 7\n1 3\n", False)
    files["dups_symmetric"] = (
        "%%MatrixMarket matrix coordinate pattern symmetric\n"
        "6 6 8\n"
        "2 1\n3 2\n3 2\n4 4\n5 3\n6 5\n6 1\n5 2\n", False)
    files["dupw_symmetric"] = (
        "%%MatrixMarket matrix coordinate real symmetric\n"
        "6 6 9\n"
        "2 1 5\n2 1 3\n3 2 1\n4 3 2\n4 1 9\n5 4 1\n6 5 4\n6 1 2\n6 1 7\n", True)
    files["dupw_general"] = (
        "%%MatrixMarket matrix coordinate integer general\n"
        "6 6 10\n"
        "1 2 4\n1 2 1\n2 3 2\n1 3 9\n3 4 1\n4 5 3\n5 6 1\n1 1 2\n6 1 1\n2 6 8\n", True)
    return files


def run(cmd, env=None):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def read_dump(path, weighted):
    with open(path, "rb") as f:
        rows, cols = np.frombuffer(f.read(8), np.int32)
        nnz = int(np.frombuffer(f.read(8), np.int64)[0])
        directed, source = np.frombuffer(f.read(8), np.int32)
        rp = np.frombuffer(f.read(4 * (rows + 1)), np.int32).copy()
        col = np.frombuffer(f.read(4 * nnz), np.int32).copy()
        val = np.frombuffer(f.read(4 * nnz), np.float32).copy() if weighted else None
    return int(rows), rp, col, val, bool(directed)


def parse_hops(text, n, source):
    d = np.zeros(n, np.int32)
    for line in text.splitlines():
        s, v, x = line.split()
        assert int(s) == source
        d[int(v)] = int(x)
    return d


def parse_weighted(text, n, source):
    d = np.zeros(n, np.float32)
    for line in text.splitlines():
        s, v, x = line.split()
        assert int(s) == source
        d[int(v)] = FLT_MAX if x == "3.40282e+38" else np.float32(float(x))
    return d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("DAWN_REFERENCE_DIR", "/root/reference"))
    args = ap.parse_args()
    import oracle as O
    from dawn_gb300 import gen
    O.build(ref_dir=args.ref, with_ref=True)
    bindir = O.REF_BIN
    work = os.path.join(HERE, "_tmp")
    os.makedirs(work, exist_ok=True)
    env1 = dict(os.environ, OMP_NUM_THREADS="1")

    graphs = {}
    for name, (text, weighted) in hand_written_inputs().items():
        p = os.path.join(HERE, name + ".mtx")
        with open(p, "w") as f:
            f.write(text)
        graphs[name] = (p, weighted)
    specs = [
        ("er_dir", gen.erdos_renyi(300, 1500, seed=21), False),
        ("rmat_sym", gen.rmat(8, 8, seed=22), False),
        ("grid_sym", gen.grid(9, 13), False),
        ("knn_sym", gen.knn(256, 4, seed=23), False),
        ("er_dir_w", gen.erdos_renyi(250, 1200, seed=24, weights=True), True),
        ("rmat_sym_w", gen.rmat(8, 8, seed=25, weights=True), True),
    ]
    for name, g, weighted in specs:
        p = os.path.join(HERE, name + ".mtx")
        gen.write_mtx(g, p, weighted=weighted)
        graphs[name] = (p, weighted)

    for name, (p, weighted) in sorted(graphs.items()):
        dump = os.path.join(work, name + ".bin")
        run([os.path.join(bindir, "ref_dump_csr"), p, str(int(weighted)), "0", dump])
        n, rp, col, val, directed = read_dump(dump, weighted)
        deg = np.diff(rp)
        nz = np.nonzero(deg)[0]
        rng = np.random.default_rng(zlib.crc32(name.encode()))
        srcs = sorted(set([int(nz[0]), int(nz[-1])] + [int(x) for x in rng.choice(nz, min(4, len(nz)))]))
        out = {"n": n, "row_ptr": rp, "col": col, "directed": directed, "weighted": weighted,
               "sources": np.array(srcs, np.int32)}
        if val is not None:
            out["val"] = val
        hop_rows, text0 = [], None
        w_rows, wtext0 = [], None
        cc_lines, ccw_lines = [], []
        for s in srcs:
            of = os.path.join(work, "out.txt")
            if os.path.exists(of):
                os.remove(of)
            run([os.path.join(bindir, "bfs_cpu"), "-i", p, "-s", str(s), "-p", "true", "-o", of])
            t = open(of).read()
            text0 = text0 if text0 is not None else t
            hop_rows.append(parse_hops(t, n, s))
            o = run([os.path.join(bindir, "cc_cpu"), "-i", p, "-s", str(s)])
            cc_lines.append([x for x in o.splitlines() if x.startswith("Closeness Centrality:")][0])
            if weighted:
                os.remove(of)
                # sssp_cpu reads the source from argv[4] (sssp_cpu.cpp:14): keep "-s S" there.
                run([os.path.join(bindir, "sssp_cpu"), "-i", p, "-s", str(s), "-p", "true", "-o", of], env=env1)
                t = open(of).read()
                wtext0 = wtext0 if wtext0 is not None else t
                w_rows.append(parse_weighted(t, n, s))
                o = run([os.path.join(bindir, "cc_cpu"), "-i", p, "-s", str(s), "-w", "true"], env=env1)
                ccw_lines.append([x for x in o.splitlines() if x.startswith("Closeness Centrality:")][0])
        out["bfs_ref"] = np.stack(hop_rows)
        out["bfs_text0"] = np.array(text0)
        out["cc_text"] = np.array(cc_lines)
        if weighted:
            out["sssp_ref"] = np.stack(w_rows)
            out["sssp_text0"] = np.array(wtext0)
            out["ccw_text"] = np.array(ccw_lines)
        # MSSP_CPU::run through the in-process capture, with a repeated source.
        if O.ref_available():
            class G:
                pass
            gg = G()
            gg.n, gg.row_ptr, gg.col, gg.m = n, rp, col, len(col)
            msrc = np.array(srcs + [srcs[0]], np.int32)
            d, _ = O.ref_mssp(gg, msrc)
            out["mssp_sources"] = msrc
            out["mssp_ref"] = d
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, n, len(col), "sources", srcs)
    shutil.rmtree(work)


if __name__ == "__main__":
    main()
