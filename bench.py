"""GTEPS benchmark of the DAWN frontier path on GB300.

Workload (one "step"): hop distances from 64 seeded sources of a symmetrised
RMAT scale-22 graph (edge factor 16, a=.57 b=.19 c=.19 d=.05, deduplicated,
self loops removed, seeded vertex relabelling), int32 CSR resident in HBM,
int32 distances (nsrc x n) written to HBM.  The graph and sources are
seeded synthetic data with the benchmark's shapes.

  value      whole-job GTEPS of the batched bitset traversal (CSR already
             resident, distances left on the device), DAWN_VARIANT_AUTO on
             the autotuned handle (the learned selector runs when the tuner
             measured it faster on this graph), CUDA events on the traversal
             stream around exactly --steps steps
  parity     the timed step's distances (and those of the heuristic and
             single-source runs) against the reference CPU path's, bit for
             bit; a mismatch exits non-zero
  e2e        the same metric through the C ABI with host buffers: per step
             dawn_graph_create from pinned host CSR + dawn_bfs into a pinned
             host array + dawn_graph_destroy
  plain      the same 64 sources through the single-source
             direction-optimising kernels, with its own roofline
  selector   learned selector against the direction heuristic, median and
             spread of repeated timings
  roofline   the dominant kernel's algorithmic bytes per launch / its
             CUDA-event launch time, from a traced replay of one step
  configs    the other benchmark configurations, one compact record each
             (weighted RMAT-22, RMAT-18 x 4,096 sources, 512 ER graphs in
             one launch), each with its parity flag against the oracle
  cpu_baseline  the reference CPU path (MSSP_CPU::run: OpenMP over sources,
             a serial queue BFS each) on all 64 sources, all host threads

Multi-GPU: sources shard across ranks (each rank its own 64 sources on its
own replica of the graph, no collective on the data path), weak scaling.
`--impl reference` times the reference CPU implementation instead.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gal-dawn_gb300"))

SCALE, EDGEFACTOR, A, B, C = 22, 16, 0.57, 0.19, 0.19
GRAPH_SEED, SOURCE_SEED, NSRC = 2022, 64, 64
METRIC = "GTEPS per GB300 (BFS/SSSP/MSSP) learned+batched vs plain; % HBM roofline"
L2_BYTES = 129 * 2 ** 20

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# headline step's kernels from one ncu capture (GB300, 2026-12-04), averaged
# over the launches of one step.  Captured with:
#   python bench.py --quick --traced --variant bitset --steps 1 --warmup 1 &&
#   ncu --nvtx --nvtx-include "dawn-step/" --clock-control none \
#       --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum \
#       --csv --log-file launches.csv python bench.py --quick --traced --variant bitset --steps 1 --warmup 1
# Keyed by kernel; a figure is reported only while the SHA-256 prefix of the
# kernel's source file matches the one it was captured on (None otherwise).
_CAPTURE = ("ncu launch list of one RMAT-22 x 64 step, bitset variant, traced form: "
            "dram__bytes_read.sum + dram__bytes_write.sum per launch")
NCU_TRAFFIC = {
    "bs_pull": {"bytes": 337.8e6, "launches": 5, "file": "gal-dawn_gb300/csrc/msbfs.cu", "sha": "8765e77b47788482",
                "source": _CAPTURE},
    "bs_emit_dist": {"bytes": 1178.3e6, "launches": 1, "file": "gal-dawn_gb300/csrc/msbfs.cu",
                     "sha": "8765e77b47788482", "source": _CAPTURE},
}
# L1/TEX global-load sectors of the level-3 pull (every in-edge unfinished)
# from `ncu --set full` of the 64-source pull (143,753,817 sectors,
# 128,306,834 in-edges; build 46d6bbfdfa9da210, whose 64-source kernels are
# the current ones): the unit the pull is bound by moves about one sector
# per SM clock, so sectors per in-edge x in-edges / (SMs x clock) bounds a
# level.
PULL_SECTORS_PER_EDGE = 143753817 / 128306834


def _source_hash(path):
    import hashlib
    try:
        with open(os.path.join(ROOT, path), "rb") as f:
            return hashlib.sha256(f.read()).hexdigest()[:16]
    except OSError:
        return None


def ncu_traffic(kernel):
    t = NCU_TRAFFIC.get(kernel)
    if not t or _source_hash(t["file"]) != t["sha"]:
        return None
    return t


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def rank_sources(g, rank):
    """The sources a rank traverses: every rank its own seeded draw of NSRC
    (the path shards by source; no rank waits on another's data)."""
    from dawn_gb300 import gen
    return gen.sources(g, NSRC, seed=SOURCE_SEED + rank)


def aggregate(torch, ms_step, edges, ws, device):
    """Whole-job figures over the ranks: the slowest rank's step time and
    the edges all ranks traversed.  `device` is where the reduction runs
    ("cuda" under NCCL, "cpu" under gloo)."""
    t = torch.tensor([float(ms_step)], dtype=torch.float64, device=device)
    e = torch.tensor([int(edges)], dtype=torch.int64, device=device)
    if ws > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(e, op=torch.distributed.ReduceOp.SUM)
    ms = float(t.item())
    total = int(e.item())
    return ms, total, total / (ms * 1e-3) / 1e9


def make_workload(scale, rank, weighted=False):
    from dawn_gb300 import gen
    t = time.time()
    g = gen.rmat(scale, EDGEFACTOR, A, B, C, seed=GRAPH_SEED, weights=weighted)
    srcs = rank_sources(g, rank)
    log(f"[bench] rmat{scale}: n={g.n} m={g.m} generated in {time.time() - t:.1f}s")
    return g, srcs


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples (every 50 ms) from the warm-up through the timed
    region and the sustained window after it."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, busy, mx, reasons = [], [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
                util = float(f[6])
            except ValueError:
                continue
            if util >= 50:
                busy.append(sm[-1])
            for name, v in zip(names, f[2:6]):
                if v.lower() == "active":
                    reasons.add(name)
        load = busy or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm), "samples_under_load": len(busy)}


def time_steps(torch, fn, steps, warmup, barrier):
    for _ in range(warmup):
        fn()
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    barrier()
    return e0.elapsed_time(e1)


def repeated(torch, fn, steps, reps):
    """Median, lowest and highest ms per step over `reps` timings of `steps`
    steps each."""
    per = [time_steps(torch, fn, steps, 1, lambda: None) / steps for _ in range(reps)]
    return statistics.median(per), min(per), max(per)


def alg_bytes(r, n, m):
    """Algorithmic HBM bytes of one kernel launch in the unit of the
    benchmark's roofline: CSR row pointers and columns read, distances
    written; visited, frontier and level words count zero (they are
    L2-sized at these graphs).

    bs_pull / bfs_pull (one bottom-up sweep): row_ptr 4(n+1) and the
      columns of the unfinished rows 4*mu.  bfs_step (single-source level
      kernel) counts as bfs_pull at pull levels (mode 1), else as bfs_push.
    bs_push_scatter / bfs_push: row_ptr + col of the frontier rows 4*(nf + mf).
    bs_emit_dist: the 64 x n distance block written once.
    """
    k = r["kernel"]
    if k == "bfs_step":  # the single-source level kernel: a pull or a push level by its mode
        k = "bfs_pull" if r.get("mode") == 1 else "bfs_push"
    if k in ("bs_pull", "bfs_pull"):
        return 4 * (n + 1) + 4 * r["unvisited_edges"]
    if k in ("bs_push_scatter", "bfs_push"):
        return 4 * (r["frontier"] + r["frontier_edges"])
    if k == "bs_emit_dist":
        return 4 * NSRC * n
    return 0


def alg_bytes_with_words(r, n, m):
    """The same, counting the bitset words each kernel must touch too (the
    pull reads every unfinished vertex's visited words and writes its
    frontier words: 16 bytes per vertex at one word per state)."""
    k = r["kernel"]
    if k == "bs_pull":
        return alg_bytes(r, n, m) + 16 * n
    if k == "bs_push_update":
        return 24 * min(r["frontier_edges"], n)
    if k == "bs_emit_dist":
        return alg_bytes(r, n, m) + 40 * n
    if k == "bs_clear":
        return 8 * n * 9
    if k == "bfs_pull":
        return alg_bytes(r, n, m) + n // 8
    return alg_bytes(r, n, m)


def kernel_roofline(recs, n, m, peak_gbs, peak_kind, skip=("bs_init", "bs_next")):
    """Per-kernel CUDA-event durations of a traced replay; the dominant
    kernel's algorithmic bytes per launch over its average launch time."""
    per = {}
    for r in recs:
        if r["kernel"] in skip:  # one-thread bookkeeping
            continue
        k = per.setdefault(r["kernel"], {"launches": 0, "ms": 0.0, "bytes": 0, "bytes_w": 0})
        k["launches"] += 1
        k["ms"] += r["ms"]
        k["bytes"] += alg_bytes(r, n, m)
        k["bytes_w"] += alg_bytes_with_words(r, n, m)
    if not per:
        return None
    total = sum(k["ms"] for k in per.values())
    dom = max(per, key=lambda k: per[k]["ms"])
    k = per[dom]
    avg_ms = k["ms"] / k["launches"]
    avg_bytes = k["bytes"] / k["launches"]
    achieved = avg_bytes / (avg_ms * 1e-3) / 1e9
    achieved_w = k["bytes_w"] / k["launches"] / (avg_ms * 1e-3) / 1e9
    traffic = ncu_traffic(dom)
    extra = {}
    if dom == "bs_pull":
        # the L1/TEX sector bound: one sector per SM per clock at the
        # maximum SM clock, sectors per in-edge from the ncu capture
        edges = sum(r["unvisited_edges"] for r in recs if r["kernel"] == dom)
        launches = k["launches"]
        sms, mhz = 152, 2070.0
        floor_ms = PULL_SECTORS_PER_EDGE * edges / launches / (sms * mhz * 1e3)
        extra["l1tex_bound"] = {"rule": "ncu sectors per in-edge x unfinished in-edges / (152 SMs x 1 sector per "
                                        "clock x 2070 MHz), per launch",
                                "floor_ms_per_launch": round(floor_ms, 4),
                                "frac": round(floor_ms / avg_ms, 4)}
    return {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak_gbs,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak_gbs, 4),
            "traffic": int(traffic["bytes"]) if traffic else None,
            "traffic_source": traffic["source"] if traffic else "not captured for this build",
            "launches_per_step": k["launches"], "avg_launch_ms": round(avg_ms, 4),
            "alg_bytes_per_launch": int(avg_bytes),
            "alg_bytes_rule": "CSR row pointers and columns read + distances written; bitset words 0",
            "with_bitset_words": {"achieved": round(achieved_w, 1), "frac": round(achieved_w / peak_gbs, 4),
                                  "alg_bytes_per_launch": int(k["bytes_w"] / k["launches"])},
            "kernel_share": {name: round(v["ms"] / total, 4) for name, v in per.items()},
            "source": "CUDA events around each kernel in a traced replay", **extra}


def traced(dg, run):
    dg.trace(True)
    run()
    dg.synchronize()
    recs = dg.trace_read()
    dg.trace(False)
    return recs


def reached_edges(d_api, deg):
    """TEPS numerator of a distance block: per source, the CSR entries whose
    tail is reached (source row included)."""
    return sum(int(deg[row >= 0].sum()) for row in d_api)


class _StdoutToStderr:
    """The reference's CPU tools print progress lines ("Start print") to
    stdout when they produce distances; they go to stderr here, so stdout
    carries only the JSON line."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        os.dup2(2, 1)

    def __exit__(self, *exc):
        try:
            import ctypes
            ctypes.CDLL(None).fflush(None)
        except OSError:
            pass
        os.dup2(self.saved, 1)
        os.close(self.saved)


def link_rates(torch, rp_h, col_h, out_h, d_dist):
    """Copy-engine rates of the host link for the e2e step's own buffers:
    the CSR in, the distance block out, and both at once on two streams
    (best of three each)."""
    d_rp = torch.empty(rp_h.shape, dtype=rp_h.dtype, device="cuda")
    d_col = torch.empty(col_h.shape, dtype=col_h.dtype, device="cuda")
    s0, s1 = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(fn):
        best = None
        for _ in range(3):
            torch.cuda.synchronize()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            dt = time.perf_counter() - t
            best = dt if best is None else min(best, dt)
        return best

    def up():
        d_rp.copy_(rp_h, non_blocking=True)
        d_col.copy_(col_h, non_blocking=True)

    def both():
        with torch.cuda.stream(s0):
            up()
        with torch.cuda.stream(s1):
            out_h.copy_(d_dist, non_blocking=True)

    bi = rp_h.numel() * 4 + col_h.numel() * 4
    bo = out_h.numel() * 4
    t_in, t_out, t_both = timed(up), timed(lambda: out_h.copy_(d_dist, non_blocking=True)), timed(both)
    del d_rp, d_col
    return {"h2d_gbs": round(bi / t_in / 1e9, 1), "d2h_gbs": round(bo / t_out / 1e9, 1),
            "both_ms": round(t_both * 1e3, 3), "in_then_out_ms": round((t_in + t_out) * 1e3, 3)}


def _cpu_impl():
    """The reference CPU path: compiled from the reference's own sources when
    that build loads here, else the oracle's restatement of it.  `run`
    returns the distance block in the reference's encoding."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    threads = os.cpu_count() or 1
    if O.ref_available():
        return O, "reference", threads, lambda g, s, want=True: O.ref_mssp(g, s, want_dist=want)[0]
    return O, "port", threads, lambda g, s, want=True: O.mssp(g, s, threads=threads, want_dist=want)[0]


def cpu_baseline(g, srcs):
    """All sources once through MSSP_CPU::run (OpenMP over sources, one
    serial queue BFS each), wall-clock timed; its distances are the parity
    reference of the timed GPU step.  Runs before the process creates its
    CUDA context: on the Grace host, first touches of fresh host pages (the
    reference allocates three n-sized arrays per source) cost several times
    more in a process that holds one."""
    O, kind, threads, run = _cpu_impl()
    # loads the library and warms the CSR pages; OpenMP's thread count is
    # process-wide state of the one runtime both libraries share, so this
    # call also leaves it at all host threads for the reference's loop
    O.mssp(g, srcs[:1], threads=threads, want_dist=False)
    with _StdoutToStderr():
        t0 = time.perf_counter()
        ref = run(g, srcs)
        dt = time.perf_counter() - t0
    want = O.hops_ref_to_api(ref, srcs)
    edges = reached_edges(want, g.degrees())
    return {"value": round(edges / dt / 1e9, 4), "unit": "GTEPS", "cores": threads, "kind": kind,
            "sample": f"all {len(srcs)} sources once ({dt:.1f} s wall, {threads} threads)",
            "call": "MSSP_CPU::run (src/algorithm/cpu/mssp.cpp:9-32)"}, want


def cpu_baseline_weighted(g, srcs):
    """SSSP_CPU::SSSP per source (src/algorithm/cpu/sssp.cpp:23-80), one
    source per thread on all host threads (the reference's own OpenMP
    relax loses updates with more than one thread per source); the result
    is the weighted parity reference."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    want = O.msssp(g, srcs, threads=threads)
    dt = time.perf_counter() - t0
    deg = g.degrees()
    edges = sum(int(deg[row != np.float32(3.4028235e38)].sum()) for row in want)
    return {"value": round(edges / dt / 1e9, 4), "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": f"all {len(srcs)} sources once ({dt:.1f} s wall, {threads} threads, one source per thread)",
            "call": "SSSP_CPU::SSSP per source"}, want, edges


def run_reference_arm(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    g, srcs = make_workload(args.scale, 0)
    O, kind, threads, run = _cpu_impl()
    # One untimed pass over all sources gives the TEPS numerator and the
    # time of a full step; a step covers every source unless the whole run
    # would pass about four minutes, then the first sources only.
    with _StdoutToStderr():
        t0 = time.perf_counter()
        want = O.hops_ref_to_api(run(g, srcs), srcs)
        full = time.perf_counter() - t0
    per_step = len(srcs)
    while per_step > 1 and (args.steps + args.warmup) * full * per_step / len(srcs) > 240:
        per_step //= 2
    sample = srcs[:per_step]
    edges = reached_edges(want[:per_step], g.degrees())
    for _ in range(args.warmup):
        run(g, sample, False)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run(g, sample, False)
    dt = time.perf_counter() - t0
    gteps = edges * args.steps / dt / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": round(gteps, 4), "unit": "GTEPS", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded RMAT)",
            "config": {"workload": f"rmat{args.scale}-ef{EDGEFACTOR}-bfs-{NSRC}src", "n": g.n, "m": g.m,
                       "sources_per_step": per_step},
            "cpu_baseline": {"value": round(gteps, 4), "unit": "GTEPS", "cores": threads, "kind": kind,
                             "sample": f"{per_step} of the {NSRC} sources per step, MSSP_CPU::run"},
            "e2e": {"value": round(gteps, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def suite_lines(torch, abi, gen, stream, rank):
    """The other workload shapes, one JSON line each (not the headline line):
    directed ER n=65,536 x 64 sources (the CPU-runnable case), weighted
    SSSP on the RMAT-22 topology x 64 sources (int32 and float32 weights),
    RMAT-18 x 4,096 sources, 512 uneven directed ER graphs (n in
    [1,024, 65,536], average degree in [4, 32], 8-64 sources each) in one
    persistent launch, BCDAWN betweenness, and two high-diameter graphs."""
    out = []

    def timed(fn, steps=3):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    # ER-64K directed, 64 sources
    g = gen.erdos_renyi(65536, 1 << 20, seed=1)
    srcs = gen.sources(g, 64, seed=2, from_lcc=False)
    with abi.Graph(g, stream=stream) as dg:
        d = torch.empty((64, g.n), dtype=torch.int32, device="cuda")
        st = dg.bfs_device(srcs, d.data_ptr(), variant=abi.VARIANT_BITSET)
        for var, name in ((abi.VARIANT_BITSET, "bitset"), (abi.VARIANT_DO, "plain")):
            ms = timed(lambda: dg.bfs_device(srcs, d.data_ptr(), variant=var, stats=False), 10)
            out.append({"suite": "er64k-directed-bfs-64src", "variant": name, "ms_per_step": round(ms, 4),
                        "gteps": round(st.edges_traversed / (ms * 1e-3) / 1e9, 2), "n": g.n, "m": g.m})
    # weighted SSSP, RMAT-22 topology, 64 sources
    g = gen.rmat(22, EDGEFACTOR, A, B, C, seed=GRAPH_SEED, weights=True)
    srcs = gen.sources(g, NSRC, seed=SOURCE_SEED)
    for w in ("i32", "f32"):
        with abi.Graph(g, weights=w, stream=stream) as dg:
            d = torch.empty((NSRC, g.n), dtype=torch.int32, device="cuda")
            for var, name in ((abi.VARIANT_AUTO, "batched (64 sources per traversal)"),
                              (abi.VARIANT_DO, "single-source")):
                st = dg.sssp_device(srcs, d.data_ptr(), variant=var)
                ms = timed(lambda: dg.sssp_device(srcs, d.data_ptr(), stats=False, variant=var), 2)
                out.append({"suite": "rmat22-sssp-64src", "weights": w, "variant": name, "ms_per_step": round(ms, 3),
                            "gteps": round(st.edges_traversed / (ms * 1e-3) / 1e9, 2), "levels": st.levels})
    del g
    # RMAT-18, 4096 sources
    g = gen.rmat(18, EDGEFACTOR, A, B, C, seed=GRAPH_SEED)
    srcs = gen.sources(g, 4096, seed=SOURCE_SEED)
    with abi.Graph(g, stream=stream) as dg:
        d = torch.empty((4096, g.n), dtype=torch.int32, device="cuda")
        st = dg.bfs_device(srcs, d.data_ptr(), variant=abi.VARIANT_BITSET)
        ms = timed(lambda: dg.bfs_device(srcs, d.data_ptr(), variant=abi.VARIANT_BITSET, stats=False), 2)
        out.append({"suite": "rmat18-bfs-4096src", "variant": "bitset", "ms_per_step": round(ms, 3),
                    "gteps": round(st.edges_traversed / (ms * 1e-3) / 1e9, 2), "n": g.n, "m": g.m})
        ms = timed(lambda: dg.bfs_device(srcs[:256], d.data_ptr(), variant=abi.VARIANT_DO, stats=False), 1)
        st2 = dg.bfs_device(srcs[:256], d.data_ptr(), variant=abi.VARIANT_DO)
        out.append({"suite": "rmat18-bfs-4096src", "variant": "plain (first 256 sources)",
                    "ms_per_step": round(ms, 3), "gteps": round(st2.edges_traversed / (ms * 1e-3) / 1e9, 2)})
        # closeness of the same 4,096 sources, reduced inside the traversal
        _, _, _, st_cc = dg.closeness(srcs, with_stats=True)
        out.append({"suite": "rmat18-closeness", "sources": 4096, "device_ms": round(st_cc.device_ms, 3),
                    "gteps": round(st_cc.edges_traversed / (st_cc.device_ms * 1e-3) / 1e9, 2),
                    "note": "no distance matrix: per-source sums from the level words"})
        allv = np.arange(g.n, dtype=np.int32)
        t0 = time.perf_counter()
        _, _, _, st_all = dg.closeness(allv, with_stats=True)
        wall = time.perf_counter() - t0
        out.append({"suite": "rmat18-closeness", "sources": int(g.n), "device_ms": round(st_all.device_ms, 3),
                    "wall_ms": round(wall * 1e3, 3),
                    "gteps": round(st_all.edges_traversed / (st_all.device_ms * 1e-3) / 1e9, 2),
                    "note": "all-vertex closeness (every vertex a source)"})
    del g, d
    # 512 independent directed ER graphs, 8-64 sources each, one persistent launch
    graphs, gsrcs = gen.er_family(ngraphs=512, seed=GRAPH_SEED)
    u, off = gen.disjoint_union(graphs)
    with abi.Graph(u, stream=stream) as dg:
        dg.set_parts(off)
        d = torch.empty(dg.multi_out_size(gsrcs), dtype=torch.int32, device="cuda")
        st = dg.multi_bfs_ptr(gsrcs, d.data_ptr(), device=True)
        ms = timed(lambda: dg.multi_bfs_ptr(gsrcs, d.data_ptr(), device=True, stats=False), 5)
        out.append({"suite": "er512-multi-graph-bfs", "variant": "one persistent launch", "ms_per_step": round(ms, 3),
                    "gteps": round(st.edges_traversed / (ms * 1e-3) / 1e9, 2), "graphs": len(graphs),
                    "sources": int(sum(len(x) for x in gsrcs)), "n_total": u.n, "m_total": u.m,
                    "levels": st.levels, "tasks": st.batches})
    del u, d
    # BCDAWN betweenness of every vertex, RMAT scale 16 (65,536 sources)
    gb = gen.rmat(16, EDGEFACTOR, A, B, C, seed=GRAPH_SEED)
    with abi.Graph(gb, stream=stream) as dg:
        dg.betweenness(np.arange(64, dtype=np.int32))
        t0 = time.perf_counter()
        _, st = dg.betweenness()
        wall = time.perf_counter() - t0
        out.append({"suite": "rmat16-betweenness-all-vertices", "sources": gb.n, "n": gb.n, "m": gb.m,
                    "device_ms": round(st.device_ms, 2), "wall_ms": round(wall * 1e3, 2),
                    "sources_per_s": round(gb.n / wall, 1), "batches": st.batches})
    # the same graphs one at a time (first 32): batched bitset per graph, and
    # the plain single-source traversal per (graph, source)
    sub = 32
    for var, name in ((abi.VARIANT_BITSET, "per-graph bitset"), (abi.VARIANT_DO, "per-graph plain")):
        tot_ms, tot_edges = 0.0, 0
        for g1, s1 in zip(graphs[:sub], gsrcs[:sub]):
            with abi.Graph(g1, stream=stream) as dg:
                d = torch.empty((len(s1), g1.n), dtype=torch.int32, device="cuda")
                st = dg.bfs_device(s1, d.data_ptr(), variant=var)
                tot_ms += timed(lambda: dg.bfs_device(s1, d.data_ptr(), variant=var, stats=False), 1)
                tot_edges += st.edges_traversed
        out.append({"suite": "er512-multi-graph-bfs", "variant": f"{name} (first {sub} graphs)",
                    "ms_per_step": round(tot_ms, 3), "gteps": round(tot_edges / (tot_ms * 1e-3) / 1e9, 2)})
    # high-diameter shapes: a 2048 x 2048 4-neighbour grid and a k = 8 kNN
    # graph on 2^21 uniform points; single-source traversals with the small-
    # frontier cluster levels on and off, and the batched traversal (levels
    # from 32 on written out directly)
    for name, g in (("grid2048x2048", gen.grid(2048, 2048)), ("knn2M-k8", gen.knn(1 << 21, 8, seed=GRAPH_SEED))):
        srcs = gen.sources(g, NSRC, seed=SOURCE_SEED)
        with abi.Graph(g, stream=stream) as dg:
            d = torch.empty((NSRC, g.n), dtype=torch.int32, device="cuda")
            for small in (1, 0):
                dg.set_option(abi.OPT_SMALL_LEVELS, small)
                st = dg.bfs_device(srcs[:2], d.data_ptr(), variant=abi.VARIANT_DO)
                ms = timed(lambda: dg.bfs_device(srcs[:2], d.data_ptr(), variant=abi.VARIANT_DO, stats=False), 1)
                out.append({"suite": f"{name}-bfs", "variant": "single-source, small-frontier cluster levels "
                            + ("on" if small else "off"), "ms_per_source": round(ms / 2, 3),
                            "gteps": round(st.edges_traversed / (ms * 1e-3) / 1e9, 3), "levels": st.levels // 2,
                            "n": g.n, "m": g.m})
            dg.set_option(abi.OPT_SMALL_LEVELS, 1)
            st = dg.bfs_device(srcs, d.data_ptr(), variant=abi.VARIANT_BITSET)
            ms = timed(lambda: dg.bfs_device(srcs, d.data_ptr(), variant=abi.VARIANT_BITSET, stats=False), 2)
            out.append({"suite": f"{name}-bfs", "variant": f"batched bitset, {NSRC} sources",
                        "ms_per_step": round(ms, 3), "ms_per_source": round(ms / NSRC, 3),
                        "gteps": round(st.edges_traversed / (ms * 1e-3) / 1e9, 3), "levels": st.levels})
        del g, d
    if rank == 0:
        for line in out:
            print(json.dumps(line), flush=True)


def quick_multi(args, torch, abi, rank):
    """--quick --graph er512: the multi-graph launch (512 uneven directed ER
    graphs, 8-64 sources each) timed alone, for profiling."""
    from dawn_gb300 import gen
    graphs, gsrcs = gen.er_family(ngraphs=512, seed=GRAPH_SEED)
    u, off = gen.disjoint_union(graphs)
    s = torch.cuda.Stream()
    torch.cuda.set_stream(s)
    with abi.Graph(u, stream=s.cuda_stream) as dg:
        dg.set_parts(off)
        d = torch.empty(dg.multi_out_size(gsrcs), dtype=torch.int32, device="cuda")
        for _ in range(args.warmup):
            dg.multi_bfs_ptr(gsrcs, d.data_ptr(), device=True, stats=False)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            dg.multi_bfs_ptr(gsrcs, d.data_ptr(), device=True, stats=False)
        e1.record()
        torch.cuda.synchronize()
        st = dg.multi_bfs_ptr(gsrcs, d.data_ptr(), device=True)
        ms = e0.elapsed_time(e1) / max(1, args.steps)
    if rank == 0:
        print(json.dumps({"quick": True, "graph": "er512", "ms_per_step": round(ms, 4), "edges": st.edges_traversed,
                          "gteps": round(st.edges_traversed / (ms * 1e-3) / 1e9, 2)}), flush=True)


def config_records(torch, abi, gen, stream, rank, g_w, srcs, peak_gbs, want_cpu, weighted_ref=None):
    """Compact records of the other benchmark configurations, each with its
    parity flag against the oracle (rank 0 checks; other ranks report
    None):

      weighted   the headline topology with int32 and float32 weights in
                 [1, 63]: 64 sources batched (min-plus, 64 per traversal)
                 and single-source; SSSP_CPU::SSSP per source as baseline
      rmat18x4096  RMAT-18, 4,096 sources, 256 per traversal (W = 4) on the
                 autotuned handle; plain = single-source on the first 256
      er512      512 directed ER graphs (n in [1,024, 65,536], average degree
                 in [4, 32], 8-64 sources each) in one persistent launch;
                 plain = single-source per graph on the first 32 graphs
    """
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    threads = os.cpu_count() or 1
    out = {}

    def timed(fn, steps):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    # --- weighted, RMAT-22 topology x 64 sources -----------------------------
    t_cfg = time.perf_counter()
    want = cpu = None
    if want_cpu:
        cpu, want_np = weighted_ref if weighted_ref else cpu_baseline_weighted(g_w, srcs)[:2]
        want = torch.from_numpy(want_np).cuda()
        del want_np
    rec = {"workload": f"rmat22-ef16-sssp-{len(srcs)}src, weights int32 and float32 in [1,63]", "cpu_baseline": cpu}
    eq = True
    for w in ("i32", "f32"):
        with abi.Graph(g_w, weights=w, stream=stream) as dg:
            dt = torch.float32 if w == "f32" else torch.int32
            d = torch.empty((len(srcs), g_w.n), dtype=dt, device="cuda")
            st = dg.sssp_device(srcs, d.data_ptr(), variant=abi.VARIANT_AUTO)
            ms_b = timed(lambda: dg.sssp_device(srcs, d.data_ptr(), stats=False, variant=abi.VARIANT_AUTO), 3)
            if want is not None:
                eq &= bool(torch.equal(_weighted_ref(torch, d, abi), want))
            ms_s = timed(lambda: dg.sssp_device(srcs, d.data_ptr(), stats=False, variant=abi.VARIANT_DO), 1)
            if want is not None:
                eq &= bool(torch.equal(_weighted_ref(torch, d, abi), want))
            e = st.edges_traversed
            rec[w] = {"batched": {"ms_per_step": round(ms_b, 3), "gteps": round(e / (ms_b * 1e-3) / 1e9, 2),
                                  "levels": st.levels},
                      "plain": {"ms_per_step": round(ms_s, 3), "gteps": round(e / (ms_s * 1e-3) / 1e9, 2)},
                      "speedup_vs_plain": round(ms_s / ms_b, 3)}
            del d
    rec["parity"] = {"equal": eq if want is not None else None, "sources": len(srcs),
                     "against": "SSSP_CPU::SSSP per source (oracle)", "checked": ["batched", "single-source"]}
    rec["wall_s"] = round(time.perf_counter() - t_cfg, 1)
    out["weighted"] = rec
    del want

    # --- RMAT-18, 4,096 sources -------------------------------------------------
    t_cfg = time.perf_counter()
    g = gen.rmat(18, EDGEFACTOR, A, B, C, seed=GRAPH_SEED)
    s4 = gen.sources(g, 4096, seed=SOURCE_SEED)
    with abi.Graph(g, stream=stream) as dg:
        tuning = dg.autotune(s4)
        d = torch.empty((4096, g.n), dtype=torch.int32, device="cuda")
        st = dg.bfs_device(s4, d.data_ptr(), variant=abi.VARIANT_AUTO)
        ms_b = timed(lambda: dg.bfs_device(s4, d.data_ptr(), variant=abi.VARIANT_AUTO, stats=False), 3)
        eq = None
        k = 512
        if want_cpu:
            ref, _, _ = O.mssp(g, s4[:k], threads=threads)
            eq = bool(torch.equal(d[:k], torch.from_numpy(O.hops_ref_to_api(ref, s4[:k])).cuda()))
        e = st.edges_traversed
        st2 = dg.bfs_device(s4[:256], d.data_ptr(), variant=abi.VARIANT_DO)
        ms_p = timed(lambda: dg.bfs_device(s4[:256], d.data_ptr(), variant=abi.VARIANT_DO, stats=False), 1)
        g_b, g_p = e / (ms_b * 1e-3) / 1e9, st2.edges_traversed / (ms_p * 1e-3) / 1e9
        out["rmat18x4096"] = {"workload": "rmat18-ef16-bfs-4096src", "n": g.n, "m": g.m,
                              "batched": {"ms_per_step": round(ms_b, 3), "gteps": round(g_b, 2),
                                          "width": tuning["bitset_width"], "learned": tuning["learned"]},
                              "plain": {"ms_per_256_sources": round(ms_p, 3), "gteps": round(g_p, 2)},
                              "speedup_vs_plain": round(g_b / g_p, 3),
                              "parity": {"equal": eq, "sources": k, "against": "MSSP_CPU::run (oracle)"},
                              "wall_s": round(time.perf_counter() - t_cfg, 1)}
        del d
    del g

    # --- 512 ER graphs, one persistent launch ------------------------------------
    t_cfg = time.perf_counter()
    graphs, gsrcs = gen.er_family(ngraphs=512, seed=GRAPH_SEED)
    u, off = gen.disjoint_union(graphs)
    with abi.Graph(u, stream=stream) as dg:
        dg.set_parts(off)
        d = torch.empty(dg.multi_out_size(gsrcs), dtype=torch.int32, device="cuda")
        st = dg.multi_bfs_ptr(gsrcs, d.data_ptr(), device=True)
        ms_b = timed(lambda: dg.multi_bfs_ptr(gsrcs, d.data_ptr(), device=True, stats=False), 5)
        eq = None
        if want_cpu:
            eq = True
            pos = 0
            for g1, s1 in zip(graphs, gsrcs):
                size = len(s1) * g1.n
                ref, _, _ = O.mssp(g1, s1, threads=threads)
                want = torch.from_numpy(O.hops_ref_to_api(ref, s1).reshape(-1)).cuda()
                eq &= bool(torch.equal(d[pos:pos + size], want))
                pos += size
        e = st.edges_traversed
        del d
    sub = 32
    ms_p, e_p = 0.0, 0
    for g1, s1 in zip(graphs[:sub], gsrcs[:sub]):
        with abi.Graph(g1, stream=stream) as dg:
            d = torch.empty((len(s1), g1.n), dtype=torch.int32, device="cuda")
            st1 = dg.bfs_device(s1, d.data_ptr(), variant=abi.VARIANT_DO)
            ms_p += timed(lambda: dg.bfs_device(s1, d.data_ptr(), variant=abi.VARIANT_DO, stats=False), 1)
            e_p += st1.edges_traversed
    g_b, g_p = e / (ms_b * 1e-3) / 1e9, e_p / (ms_p * 1e-3) / 1e9
    out["er512"] = {"workload": "512 directed ER graphs, 8-64 sources each, one persistent launch",
                    "graphs": len(graphs), "sources": int(sum(len(x) for x in gsrcs)),
                    "batched": {"ms_per_step": round(ms_b, 3), "gteps": round(g_b, 2)},
                    "plain": {"graphs": sub, "ms": round(ms_p, 3), "gteps": round(g_p, 2)},
                    "speedup_vs_plain": round(g_b / g_p, 3),
                    "parity": {"equal": eq, "parts": len(graphs), "against": "MSSP_CPU::run per graph (oracle)"},
                    "wall_s": round(time.perf_counter() - t_cfg, 1)}
    return out


def _weighted_ref(torch, d, abi):
    """Device distances in the reference's float encoding (FLT_MAX for
    unreachable)."""
    if d.dtype == torch.float32:
        return d
    f = d.to(torch.float32)
    return torch.where(d == abi.INT32_MAX, torch.tensor(float(abi.FLT_MAX), device=d.device), f)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="dawn", choices=["dawn", "reference"])
    ap.add_argument("--scale", type=int, default=SCALE)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and parity legs")
    ap.add_argument("--no-configs", action="store_true", help="skip the other configurations' records")
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--reps", type=int, default=5, help="repeats of the selector-vs-heuristic timing")
    ap.add_argument("--sustain-s", type=float, default=1.5,
                    help="seconds of the headline step run after the timed region for the clock record")
    ap.add_argument("--quick", action="store_true",
                    help="only the device-resident timing (profiling runs); prints a short JSON line")
    ap.add_argument("--traced", action="store_true",
                    help="with --quick: run the steps level by level, launching only the kernels each level uses")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner before the timed steps")
    ap.add_argument("--variant", default="bitset", choices=["bitset", "learned", "do", "push", "sssp", "sssp-single"],
                    help="--quick only: the traversal to run (sssp: batched weighted, int32 weights)")
    ap.add_argument("--graph", default="rmat", choices=["rmat", "grid1024", "grid2048", "knn2M", "er64k", "er512"],
                    help="--quick only: rmat (of --scale), a 4-neighbour grid, a k = 8 kNN graph on 2^21 points, "
                         "the directed ER graph of 65,536 vertices and 2^20 edges, "
                         "or the 512 uneven ER graphs in one multi-graph launch")
    ap.add_argument("--sources", type=int, default=NSRC, help="--quick only: sources per step")
    ap.add_argument("--suite", action="store_true",
                    help="also time the other workload shapes (one JSON line each, before the main line)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)

    ws, rank, local = dist_env()
    # The reference CPU path first, before this process creates a CUDA
    # context: its distances are the parity reference of every GPU run
    # below (rank 0; other ranks meet it at the process-group set-up).
    g = srcs = None
    cpu = want_np = weighted_ref = None
    if not args.quick:
        # weights drawn too: the weighted configuration shares the topology
        g, srcs = make_workload(args.scale, rank, weighted=True)
        if rank == 0 and not args.no_cpu:
            cpu, want_np = cpu_baseline(g, srcs)
            if not args.no_configs:
                weighted_ref = cpu_baseline_weighted(g, srcs)[:2]
    import torch
    from dawn_gb300 import abi
    torch.cuda.set_device(local)
    barrier = lambda: None  # noqa: E731
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        barrier = dist.barrier
    if args.suite:
        from dawn_gb300 import gen as _gen
        _s = torch.cuda.Stream()
        torch.cuda.set_stream(_s)
        suite_lines(torch, abi, _gen, _s.cuda_stream, rank)
    if args.quick and args.graph == "er512":
        return quick_multi(args, torch, abi, rank)
    if args.quick and args.graph != "rmat":
        from dawn_gb300 import gen as _gen
        g = {"grid1024": lambda: _gen.grid(1024, 1024), "grid2048": lambda: _gen.grid(2048, 2048),
             "knn2M": lambda: _gen.knn(1 << 21, 8, seed=GRAPH_SEED),
             "er64k": lambda: _gen.erdos_renyi(65536, 1 << 20, seed=1)}[args.graph]()
        if args.graph == "er64k":  # the suite's sources for this graph
            srcs = _gen.sources(g, NSRC, seed=2, from_lcc=False)
        else:
            srcs = _gen.sources(g, NSRC, seed=SOURCE_SEED + rank)
    elif args.quick:
        g, srcs = make_workload(args.scale, rank, weighted=args.variant.startswith("sssp"))
    if args.quick:
        srcs = srcs[:args.sources]
    # A dedicated stream: the library launches on it and torch's events
    # record on it (the legacy default stream has handle 0, which the C ABI
    # reads as "library-owned stream").
    tstream = torch.cuda.Stream()
    torch.cuda.set_stream(tstream)
    stream = tstream.cuda_stream
    peak_gbs, peak_kind = peaks()

    dg = abi.Graph(g, stream=stream)
    d_dist = torch.empty((NSRC, g.n), dtype=torch.int32, device="cuda")
    if args.quick:
        # Profiling form: the same traversal as a bench step (handle tuned
        # first, untimed), with the measured steps inside an NVTX range
        # "dawn-step" so a profiler can keep to exactly those launches.
        if args.variant.startswith("sssp"):
            dg.close()
            dg = abi.Graph(g, weights="i32", stream=stream)
            var = abi.VARIANT_AUTO if args.variant == "sssp" else abi.VARIANT_DO
            run = lambda st=False: dg.sssp_device(srcs, d_dist.data_ptr(), variant=var, stats=st)  # noqa: E731
        else:
            var = {"bitset": abi.VARIANT_BITSET, "learned": abi.VARIANT_LEARNED, "do": abi.VARIANT_DO,
                   "push": abi.VARIANT_PUSH}[args.variant]
            if not args.no_tune and var in (abi.VARIANT_BITSET, abi.VARIANT_LEARNED):
                dg.autotune(srcs)
            run = lambda st=False: dg.bfs_device(srcs, d_dist.data_ptr(), variant=var, stats=st)  # noqa: E731
        for _ in range(args.warmup):
            run()
        torch.cuda.synchronize()
        dg.trace(args.traced)

        def quick():
            torch.cuda.nvtx.range_push("dawn-step")
            run()
            torch.cuda.nvtx.range_pop()
        ms = time_steps(torch, quick, args.steps, 0, barrier) / max(1, args.steps)
        recs = dg.trace_read() if args.traced else []
        dg.trace(False)
        for r in recs:
            log("[trace] run %d level %d mode %d %-16s frontier %9d fedges %11d unfinished_edges %11d  %.3f ms" % (
                r["run"], r["level"], r["mode"], r["kernel"], r["frontier"], r["frontier_edges"],
                r["unvisited_edges"], r["ms"]))
        st = run(True)
        if rank == 0:
            print(json.dumps({"quick": True, "variant": args.variant, "traced": args.traced, "graph": args.graph,
                              "scale": args.scale, "sources": len(srcs),
                              "ms_per_step": round(ms, 4), "edges": st.edges_traversed,
                              "gteps": round(st.edges_traversed / (ms * 1e-3) / 1e9, 2),
                              "kernels": len(recs)}), flush=True)
        dg.close()
        return

    st0 = dg.bfs_device(srcs, d_dist.data_ptr(), variant=abi.VARIANT_BITSET, stats=True)
    edges = st0.edges_traversed
    want = None
    if want_np is not None:
        want = torch.from_numpy(want_np).cuda()
        del want_np
    checks = {}

    def check(name):
        if want is not None:
            torch.cuda.synchronize()
            checks[name] = bool(torch.equal(d_dist, want))

    check("untuned bitset")
    # learned + batched: the autotuner sets the handle's speed options first
    # (untimed, once per graph); AUTO then runs the batched traversal with the
    # learned selector when the tuner measured it faster, else the heuristic
    tuning = None
    if not args.no_tune:
        tuning = dg.autotune(srcs)
    var = abi.VARIANT_AUTO
    step = lambda: dg.bfs_device(srcs, d_dist.data_ptr(), variant=var, stats=False)  # noqa
    st = dg.bfs_device(srcs, d_dist.data_ptr(), variant=var, stats=True)

    clocks = Clocks(local)
    clocks.start()
    ms = time_steps(torch, step, args.steps, args.warmup, barrier)
    check("headline (timed step)")
    # a sustained window of the same step right after, so the clock record
    # covers more than the short timed region
    n_sus = max(args.steps, int(args.sustain_s * 1e3 / max(ms / args.steps, 1e-3)))
    ms_sus = time_steps(torch, step, n_sus, 0, barrier) / n_sus
    clk = clocks.stop()
    # the slowest rank's time, the edges of all ranks
    ms_step, _, value = aggregate(torch, ms / args.steps, edges, ws, "cuda")

    # learned selector against the direction heuristic, repeated
    sel = {}
    for name, v in (("learned", abi.VARIANT_LEARNED), ("heuristic", abi.VARIANT_BITSET)):
        fn = lambda v=v: dg.bfs_device(srcs, d_dist.data_ptr(), variant=v, stats=False)  # noqa: E731
        med, lo, hi = repeated(torch, fn, args.steps, args.reps)
        check(f"batched {name}")
        sel[name] = {"ms_median": round(med, 4), "ms_min": round(lo, 4), "ms_max": round(hi, 4),
                     "gteps_median": round(edges / (med * 1e-3) / 1e9, 2)}
    spread = max(sel["learned"]["ms_max"] - sel["learned"]["ms_min"],
                 sel["heuristic"]["ms_max"] - sel["heuristic"]["ms_min"])
    sel["learned_gain"] = round(sel["heuristic"]["ms_median"] / sel["learned"]["ms_median"] - 1.0, 4)
    sel["beats_heuristic_beyond_spread"] = sel["heuristic"]["ms_median"] - sel["learned"]["ms_median"] > spread
    sel["reps"] = args.reps
    sel["auto_uses_selector"] = bool(tuning["learned"]) if tuning else False

    # plain single-source direction-optimising kernels, same sources
    step_plain = lambda: dg.bfs_device(srcs, d_dist.data_ptr(), variant=abi.VARIANT_DO, stats=False)  # noqa
    ms_plain = time_steps(torch, step_plain, args.plain_steps, 1, barrier) / args.plain_steps
    check("plain single-source")
    reached = int((d_dist >= 0).sum().item())
    plain_bytes = 4 * edges + 4 * (reached + NSRC) + 4 * g.n * NSRC
    plain_ach = plain_bytes / (ms_plain * 1e-3) / 1e9
    plain = {"value": round(edges / (ms_plain * 1e-3) / 1e9, 3), "unit": "GTEPS",
             "ms_per_step": round(ms_plain, 3), "variant": "single-source push/pull (direction-optimising)",
             "roofline": {"bound": "hbm", "achieved": round(plain_ach, 1), "peak": peak_gbs, "peak_kind": peak_kind,
                          "unit": "GB/s", "frac": round(plain_ach / peak_gbs, 4), "alg_bytes_per_step": plain_bytes,
                          "alg_bytes_rule": "per source 4*m_r + 4*(n_r + 1) + 4*n (reached edges, reached "
                                            "vertices, distance row)"}}
    recs_plain = traced(dg, lambda: dg.bfs_device(srcs[:2], d_dist.data_ptr(), variant=abi.VARIANT_DO, stats=False))
    for r in recs_plain:
        log("[trace-plain] src %d level %d mode %d %-10s frontier %9d fedges %11d unvisited_edges %11d %.3f ms"
            % (r["run"], r["level"], r["mode"], r["kernel"], r["frontier"], r["frontier_edges"],
               r["unvisited_edges"], r["ms"]))
    plain["roofline"]["kernel"] = kernel_roofline(recs_plain, g.n, g.m, peak_gbs, peak_kind,
                                                  skip=("bfs_init", "bfs_decide", "bs_init", "bs_next"))

    recs = traced(dg, lambda: dg.bfs_device(srcs, d_dist.data_ptr(), variant=var, stats=False))
    check("traced replay")
    for r in recs:
        log("[trace] run %d level %d mode %d %-16s frontier %9d fedges %11d unfinished_edges %11d  %.3f ms" % (
            r["run"], r["level"], r["mode"], r["kernel"], r["frontier"], r["frontier_edges"],
            r["unvisited_edges"], r["ms"]))
    roof = kernel_roofline(recs, g.n, g.m, peak_gbs, peak_kind)
    step_bytes = 4 * g.m + 4 * (g.n + 1) + NSRC * 4 * g.n
    roof["step_alg_bytes"] = step_bytes
    roof["step_achieved"] = round(step_bytes / (ms_step * 1e-3) / 1e9, 1)
    roof["step_frac"] = round(step_bytes / (ms_step * 1e-3) / 1e9 / peak_gbs, 4)

    # end to end through the C ABI with pinned host buffers, and the host
    # link's own rates for the same bytes (a step moves the CSR in and the
    # distance block out; the link carries one direction at a time here:
    # both copies at once take as long as the two in turn)
    rp_h = torch.from_numpy(g.row_ptr).pin_memory()
    col_h = torch.from_numpy(g.col).pin_memory()
    out_h = torch.empty((NSRC, g.n), dtype=torch.int32).pin_memory()
    phases = {"create_ms": 0.0, "bfs_ms": 0.0, "destroy_ms": 0.0}

    def e2e_step(record=False):
        t0 = time.perf_counter()
        h = abi.Graph(raw=dict(n=g.n, m=g.m, row_ptr=rp_h.data_ptr(), col=col_h.data_ptr(), symmetric=True,
                               stream=stream))
        if tuning is not None:
            h.autotune(srcs, use_cache=True)  # the graph class's tuned settings, nothing measured
        t1 = time.perf_counter()
        h.bfs_host_ptr(srcs, out_h.data_ptr(), variant=var)
        t2 = time.perf_counter()
        h.close()
        t3 = time.perf_counter()
        if record:
            phases["create_ms"] += (t1 - t0) * 1e3
            phases["bfs_ms"] += (t2 - t1) * 1e3
            phases["destroy_ms"] += (t3 - t2) * 1e3

    e2e_step()
    torch.cuda.synchronize()
    if want is not None:
        checks["e2e (host buffers)"] = bool(torch.equal(out_h, want.cpu()))
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_step(record=True)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.e2e_steps
    e2e_ms, _, e2e_gteps = aggregate(torch, e2e_ms, edges, ws, "cuda")
    h2d = 4 * (g.n + 1) + 4 * g.m + 4 * NSRC
    d2h = 4 * NSRC * g.n
    link = link_rates(torch, rp_h, col_h, out_h, d_dist)
    bound_ms = h2d / (link["h2d_gbs"] * 1e6) + d2h / (link["d2h_gbs"] * 1e6) + ms_step
    e2e = {"value": round(e2e_gteps, 3), "unit": "GTEPS", "ms_per_step": round(e2e_ms, 3),
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "phases_ms": {k: round(v / args.e2e_steps, 3) for k, v in phases.items()},
           "call": "dawn_graph_create(pinned host CSR) + dawn_bfs(pinned host dist) + dawn_graph_destroy",
           "link": link, "bound_ms": round(bound_ms, 3), "frac_of_bound": round(bound_ms / e2e_ms, 4),
           "bound_rule": "CSR in at the measured host-to-device rate + distances out at the measured "
                         "device-to-host rate + the device-resident step"}
    del want
    dg.close()
    del d_dist

    configs = None
    if not args.no_configs:
        from dawn_gb300 import gen as _gen
        configs = config_records(torch, abi, _gen, stream, rank, g, srcs, peak_gbs,
                                 want_cpu=rank == 0 and not args.no_cpu, weighted_ref=weighted_ref)
        weighted_ref = None

    parity = None
    if checks:
        parity = {"config": f"rmat{args.scale} x {NSRC} sources", "equal": all(checks.values()),
                  "sources": NSRC, "against": cpu["kind"] + " MSSP_CPU::run", "checked": checks}
    # Kernels one graph-mode step launches: clear and init, the four body
    # kernels (pull, push scatter, push update, decide) at every level (those
    # of the other direction return at once), emit and next.
    levels = len({(r["run"], r["level"]) for r in recs if r["level"] >= 1})
    launches = 2 + 4 * levels + 2
    line = {"metric": METRIC, "value": round(value, 3), "unit": "GTEPS", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded RMAT)",
            "config": {"workload": f"rmat{args.scale}-ef{EDGEFACTOR}-bfs-{NSRC}src-batched-auto", "n": g.n,
                       "m": g.m,
                       "sources": NSRC, "edges_traversed_per_step": edges,
                       "l2": "inputs larger than L2 (CSR %.0f MB, distances %.0f MB per step)" % (
                           (4 * g.m + 4 * g.n) / 2 ** 20, 4 * NSRC * g.n / 2 ** 20),
                       "parallelism": f"sources sharded, {ws} replica(s)"},
            "parity": parity, "clocks": clk,
            "sustained": {"steps": n_sus, "ms_per_step": round(ms_sus, 4),
                          "value": round(edges / (ms_sus * 1e-3) / 1e9, 3)},
            "e2e": e2e, "plain": plain, "selector": sel, "tuning": tuning,
            "speedup_vs_plain": round(value / plain["value"], 3) if plain["value"] else None,
            "roofline": roof, "cpu_baseline": cpu, "configs": configs, "gpu_launches": launches * args.steps,
            "levels_per_step": st.levels, "push_levels": st.push_levels, "pull_levels": st.pull_levels}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    bad = [k for k, v in checks.items() if not v]
    if configs:
        bad += [k for k, v in configs.items() if v.get("parity", {}).get("equal") is False]
    if bad:
        log("[bench] PARITY MISMATCH: " + ", ".join(bad))
        sys.exit(3)


if __name__ == "__main__":
    main()
