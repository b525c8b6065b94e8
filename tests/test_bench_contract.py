"""Host-side pieces of bench.py's JSON line, checked on CPU: the roofline's
traffic comes from the committed ncu launch list of the headline workload,
and the algorithmic bytes per launch follow the per-kernel formulas."""

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path[:0] = [ROOT]

import bench  # noqa: E402


def test_profiled_traffic_reads_the_committed_launch_list():
    t = bench.profiled_traffic("bs_pull", 22)
    assert t is not None
    # the pull reads more than its algorithmic bytes (315 MB per launch on
    # RMAT-22 x 64) and far less than the whole step's traffic
    assert 3.0e8 < t < 1.0e9
    assert bench.profiled_traffic("bs_pull", 20) is None
    assert bench.profiled_traffic("no_such_kernel", 22) is None


def test_alg_bytes_per_kernel():
    n, m = 1000, 16000
    pull = {"kernel": "bs_pull", "unvisited_edges": 5000, "frontier": 10, "frontier_edges": 50}
    assert bench.alg_bytes(pull, n, m) == 4 * (n + 1) + 16 * n + 4 * 5000
    scatter = {"kernel": "bs_push_scatter", "frontier": 10, "frontier_edges": 50, "unvisited_edges": 0}
    assert bench.alg_bytes(scatter, n, m) == 4 * 60
    update = {"kernel": "bs_push_update", "frontier": 10, "frontier_edges": 5000, "unvisited_edges": 0}
    assert bench.alg_bytes(update, n, m) == 24 * n  # bounded by the vertex count
    emit = {"kernel": "bs_emit_dist", "frontier": 0, "frontier_edges": 0, "unvisited_edges": 0}
    assert bench.alg_bytes(emit, n, m) == 4 * bench.NSRC * n + 40 * n
    assert bench.alg_bytes({"kernel": "bs_decide"}, n, m) == 0
