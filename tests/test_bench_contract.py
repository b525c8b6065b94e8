"""Host-side pieces of bench.py's JSON line, checked on CPU: the algorithmic
bytes per launch follow the benchmark's rule (CSR reads and distance writes;
bitset words count zero), the roofline record is built from per-launch
durations, and an ncu traffic figure is reported only for the build it was
captured on."""

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path[:0] = [ROOT]

import bench  # noqa: E402


def test_alg_bytes_per_kernel():
    n, m = 1000, 16000
    pull = {"kernel": "bs_pull", "unvisited_edges": 5000, "frontier": 10, "frontier_edges": 50}
    assert bench.alg_bytes(pull, n, m) == 4 * (n + 1) + 4 * 5000
    assert bench.alg_bytes_with_words(pull, n, m) == 4 * (n + 1) + 16 * n + 4 * 5000
    single = dict(pull, kernel="bfs_pull")
    assert bench.alg_bytes(single, n, m) == 4 * (n + 1) + 4 * 5000
    assert bench.alg_bytes(dict(pull, kernel="bfs_step", mode=1), n, m) == 4 * (n + 1) + 4 * 5000
    assert bench.alg_bytes(dict(pull, kernel="bfs_step", mode=0), n, m) == 4 * (10 + 50)
    scatter = {"kernel": "bs_push_scatter", "frontier": 10, "frontier_edges": 50, "unvisited_edges": 0}
    assert bench.alg_bytes(scatter, n, m) == 4 * 60
    update = {"kernel": "bs_push_update", "frontier": 10, "frontier_edges": 5000, "unvisited_edges": 0}
    assert bench.alg_bytes(update, n, m) == 0
    assert bench.alg_bytes_with_words(update, n, m) == 24 * n  # bounded by the vertex count
    emit = {"kernel": "bs_emit_dist", "frontier": 0, "frontier_edges": 0, "unvisited_edges": 0}
    assert bench.alg_bytes(emit, n, m) == 4 * bench.NSRC * n
    assert bench.alg_bytes({"kernel": "bs_decide"}, n, m) == 0


def test_kernel_roofline_picks_the_dominant_kernel():
    n, m = 1000, 16000
    recs = [{"kernel": "bs_pull", "unvisited_edges": 8000, "frontier": 0, "frontier_edges": 0, "ms": 0.002},
            {"kernel": "bs_pull", "unvisited_edges": 2000, "frontier": 0, "frontier_edges": 0, "ms": 0.002},
            {"kernel": "bs_push_scatter", "unvisited_edges": 0, "frontier": 5, "frontier_edges": 95, "ms": 0.001},
            {"kernel": "bs_init", "unvisited_edges": 0, "frontier": 0, "frontier_edges": 0, "ms": 0.5}]
    r = bench.kernel_roofline(recs, n, m, 1000.0, "measured")
    assert r["kernel"] == "bs_pull" and r["launches_per_step"] == 2
    per_launch = (4 * (n + 1) * 2 + 4 * 10000) / 2
    assert r["alg_bytes_per_launch"] == int(per_launch)
    assert abs(r["achieved"] - per_launch / 2e-6 / 1e9) < 0.1
    assert abs(r["frac"] - r["achieved"] / 1000.0) < 1e-3
    assert "bs_init" not in r["kernel_share"]


def test_traffic_only_for_the_captured_build(monkeypatch):
    monkeypatch.setattr(bench, "NCU_TRAFFIC", {
        "bs_pull": {"bytes": 4.0e8, "file": "bench.py", "sha": bench._source_hash("bench.py"), "source": "x"},
        "bs_emit_dist": {"bytes": 1.0e9, "file": "bench.py", "sha": "0" * 16, "source": "y"}})
    assert bench.ncu_traffic("bs_pull")["bytes"] == 4.0e8
    assert bench.ncu_traffic("bs_emit_dist") is None  # captured on another build
    assert bench.ncu_traffic("bs_push_update") is None


def test_committed_traffic_matches_the_committed_kernels():
    # a kernel file changed without a new ncu capture would report traffic
    # null in the bench line: the capture and its constants go with the change
    for kernel, t in bench.NCU_TRAFFIC.items():
        assert bench.ncu_traffic(kernel) is not None, (kernel, t["file"], bench._source_hash(t["file"]), t["sha"])


def test_reached_edges():
    import numpy as np
    deg = np.array([3, 1, 0, 2], np.int64)
    d = np.array([[0, 1, -1, 2], [-1, -1, 0, -1]], np.int32)
    assert bench.reached_edges(d, deg) == 3 + 1 + 2 + 0
