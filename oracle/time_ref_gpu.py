"""ORACLE — test infrastructure only.

Times the reference's own single-source GPU path on this GPU, next to this
library's, on the benchmark graph (symmetrised RMAT scale 22, edge factor
16, a/b/c 0.57/0.19/0.19, seed 2022, integer weights in [1, 63] as float32;
the first sources of the benchmark's 64-source draw, seed 64):

  - SOVM + BFS_GPU::kernel (src/algorithm/gpu/bfs.cu:9-105) and GOVM +
    SSSP_GPU::kernel (src/algorithm/gpu/sssp.cu:30-129), unmodified,
    compiled for sm_103a by ``make -C oracle ref-gpu`` (ref_gpu_shim.cu);
  - before any time is quoted, every source's distances are compared with
    the oracle (MSSP_CPU::run restated for hops, SSSP_CPU::SSSP restated
    per source for weights).  The reference's GPU loops leave the source's
    own entry at a path length (it starts as "unvisited" and is reached
    again through a neighbour), so the source entry is reported apart;
    every other vertex must match;
  - this library's single-source kernels (variant DO) and batched
    traversal (AUTO, 64 sources at once) on the same graph, device-side,
    CUDA events.

The reference's time is its own (the host clock around its level loop,
which includes its flag reads every third / fifth level); ours is CUDA
events around the traversals.  One JSON line per workload on stdout.

    python oracle/time_ref_gpu.py [--scale 22] [--bfs-sources 8] [--sssp-sources 4]
"""

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [HERE, os.path.join(ROOT, "gal-dawn_gb300")]

import oracle as O  # noqa: E402

LIB = os.path.join(HERE, "_ref", "libdawn_ref_gpu.so")
BLOCK = 1024  # graph.block_size in the reference's GPU drivers (algorithm/gpu/*/*.cu)
FLT_MAX = np.float32(np.finfo(np.float32).max)


class _StdoutToStderr:
    """The reference's loops print "Start print" before handing back their
    distances; that goes to stderr, so stdout carries only JSON."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        os.dup2(2, 1)

    def __exit__(self, *exc):
        ctypes.CDLL(None).fflush(None)
        os.dup2(self.saved, 1)
        os.close(self.saved)


def load():
    ref = O.reference_dir()
    if ref is not None:
        subprocess.run(["make", "-s", "-C", HERE, "ref-gpu", f"REF={ref}"], check=True)
    if not os.path.exists(LIB):
        return None
    L = ctypes.CDLL(LIB)
    P, I32, I64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    L.ref_gpu_open.restype = P
    L.ref_gpu_open.argtypes = [P, P, P, I32, I64, I32]
    L.ref_gpu_close.argtypes = [P]
    L.ref_gpu_bfs.argtypes = [P, I32, P, ctypes.POINTER(ctypes.c_float)]
    L.ref_gpu_sssp.argtypes = [P, I32, P, ctypes.POINTER(ctypes.c_float)]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def compare(got, want, source, unreached_got, unreached_want):
    """Mismatches over every vertex but the source, and the source's entry."""
    mask = np.ones(got.shape[0], bool)
    mask[source] = False
    g = np.where(got == unreached_got, unreached_want, got)
    bad = int(np.count_nonzero(g[mask] != want[mask]))
    return bad, got[source].item()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--bfs-sources", type=int, default=8)
    ap.add_argument("--sssp-sources", type=int, default=4)
    args = ap.parse_args()

    L = load()
    if L is None:
        print(json.dumps({"reference_gpu": "unavailable", "why": "no reference sources to compile"}))
        return 0
    from dawn_gb300 import abi, gen
    g = gen.rmat(args.scale, 16, 0.57, 0.19, 0.19, seed=2022, weights=True)
    srcs = gen.sources(g, 64, seed=64)
    threads = os.cpu_count() or 1
    kb, ks = args.bfs_sources, args.sssp_sources
    deg = g.degrees()

    # the oracle first (host threads), then the GPU
    want_h, edges_h, _ = O.mssp(g, srcs[:kb], threads=threads)
    want_w = O.msssp(g, srcs[:ks], threads=threads)
    edges_w = [int(deg[want_w[i] != FLT_MAX].sum()) for i in range(ks)]
    edges_h_per = [int(deg[want_h[i] != 0].sum()) + int(deg[srcs[i]]) for i in range(kb)]

    h = L.ref_gpu_open(_p(g.row_ptr), _p(g.col), _p(g.w_f32), g.n, g.m, BLOCK)
    if not h:
        raise RuntimeError("ref_gpu_open failed")
    ms = ctypes.c_float()
    rec_h = {"workload": f"rmat{args.scale}-ef16 single-source BFS, sources {kb} of the benchmark's 64",
             "reference": "SOVM + BFS_GPU::kernel, sm_103a, block 1024"}
    rec_w = {"workload": f"rmat{args.scale}-ef16 single-source SSSP (float32 weights in [1,63]), "
                         f"sources {ks} of the benchmark's 64",
             "reference": "GOVM + SSSP_GPU::kernel, sm_103a, block 1024"}
    try:
        d = np.zeros(g.n, np.int32)
        with _StdoutToStderr():
            rc = L.ref_gpu_bfs(h, int(srcs[0]), _p(d), ctypes.byref(ms))  # warm-up (module load)
        if rc != 0:
            raise RuntimeError(f"ref_gpu_bfs: {rc}")
        times, bad, src_entries = [], [], []
        for i in range(kb):
            with _StdoutToStderr():
                rc = L.ref_gpu_bfs(h, int(srcs[i]), _p(d), ctypes.byref(ms))
            if rc != 0:
                raise RuntimeError(f"ref_gpu_bfs: {rc}")
            times.append(ms.value)
            b, se = compare(d, want_h[i], int(srcs[i]), 0, 0)
            bad.append(b)
            src_entries.append(int(se))
        rec_h["reference_ms_per_source"] = round(float(np.median(times)), 3)
        rec_h["reference_ms"] = [round(t, 3) for t in times]
        rec_h["reference_mismatches_excl_source"] = bad
        rec_h["reference_source_entry"] = src_entries
        rec_h["reference_gteps"] = round(sum(edges_h_per) / (sum(times) * 1e-3) / 1e9, 3)

        dw = np.zeros(g.n, np.float32)
        times, bad, src_entries = [], [], []
        for i in range(ks):
            with _StdoutToStderr():
                rc = L.ref_gpu_sssp(h, int(srcs[i]), _p(dw), ctypes.byref(ms))
            if rc != 0:
                raise RuntimeError(f"ref_gpu_sssp: {rc}")
            times.append(ms.value)
            b, se = compare(dw, want_w[i], int(srcs[i]), FLT_MAX, FLT_MAX)
            bad.append(b)
            src_entries.append(float(se))
        rec_w["reference_ms_per_source"] = round(float(np.median(times)), 3)
        rec_w["reference_ms"] = [round(t, 3) for t in times]
        rec_w["reference_mismatches_excl_source"] = bad
        rec_w["reference_source_entry"] = src_entries
        rec_w["reference_gteps"] = round(sum(edges_w) / (sum(times) * 1e-3) / 1e9, 3)
    finally:
        L.ref_gpu_close(h)

    import torch

    # the library launches on this stream and the events record on it
    tstream = torch.cuda.Stream()
    torch.cuda.set_stream(tstream)
    stream = tstream.cuda_stream

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    want_api = O.hops_ref_to_api(want_h, srcs[:kb])
    with abi.Graph(g, stream=stream) as dg:
        d = torch.empty((64, g.n), dtype=torch.int32, device="cuda")
        st = dg.bfs_device(srcs[:kb], d.data_ptr(), variant=abi.VARIANT_DO)
        ok = bool(np.array_equal(d[:kb].cpu().numpy(), want_api))
        t1 = timed(lambda: dg.bfs_device(srcs[:kb], d.data_ptr(), variant=abi.VARIANT_DO, stats=False), 3) / kb
        stb = dg.bfs_device(srcs, d.data_ptr(), variant=abi.VARIANT_AUTO)
        ok &= bool(np.array_equal(d[:kb].cpu().numpy(), want_api))
        tb = timed(lambda: dg.bfs_device(srcs, d.data_ptr(), variant=abi.VARIANT_AUTO, stats=False), 5)
        del d
    rec_h["ours_single_source_ms_per_source"] = round(t1, 4)
    rec_h["ours_single_source_gteps"] = round(st.edges_traversed / (t1 * kb * 1e-3) / 1e9, 2)
    rec_h["ours_batched_ms_per_source"] = round(tb / 64, 5)
    rec_h["ours_batched_gteps"] = round(stb.edges_traversed / (tb * 1e-3) / 1e9, 1)
    rec_h["ours_equal_oracle"] = ok
    rec_h["single_source_speedup"] = round(rec_h["reference_ms_per_source"] / t1, 1)
    print(json.dumps(rec_h), flush=True)

    with abi.Graph(g, weights="f32", stream=stream) as dg:
        d = torch.empty((64, g.n), dtype=torch.float32, device="cuda")
        st = dg.sssp_device(srcs[:ks], d.data_ptr(), variant=abi.VARIANT_DO)
        ok = bool(np.array_equal(d[:ks].cpu().numpy(), want_w))
        t1 = timed(lambda: dg.sssp_device(srcs[:ks], d.data_ptr(), stats=False, variant=abi.VARIANT_DO), 3) / ks
        stb = dg.sssp_device(srcs, d.data_ptr(), variant=abi.VARIANT_AUTO)
        ok &= bool(np.array_equal(d[:ks].cpu().numpy(), want_w))
        tb = timed(lambda: dg.sssp_device(srcs, d.data_ptr(), stats=False, variant=abi.VARIANT_AUTO), 3)
        del d
    rec_w["ours_single_source_ms_per_source"] = round(t1, 4)
    rec_w["ours_single_source_gteps"] = round(st.edges_traversed / (t1 * ks * 1e-3) / 1e9, 2)
    rec_w["ours_batched_ms_per_source"] = round(tb / 64, 4)
    rec_w["ours_batched_gteps"] = round(stb.edges_traversed / (tb * 1e-3) / 1e9, 1)
    rec_w["ours_equal_oracle"] = ok
    rec_w["single_source_speedup"] = round(rec_w["reference_ms_per_source"] / t1, 1)
    print(json.dumps(rec_w), flush=True)
    return 0


if __name__ == "__main__":
    t0 = time.time()
    rc = main()
    print(f"[time_ref_gpu] {time.time() - t0:.1f} s", file=sys.stderr)
    sys.exit(rc)
