"""The reference's own GPU kernels (SOVM, GOVM and their level loops) build
for sm_103a from their unmodified sources, through oracle/ref_gpu_shim.cu.
oracle/time_ref_gpu.py times them on a GPU next to this library's kernels,
after checking their distances against the oracle.  This test needs no
GPU: it builds the shim, checks its C entry points, and checks that opening
a handle without a device fails with NULL rather than an exception across
the C boundary.  Skipped where the reference sources are absent."""

import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.join(os.path.dirname(HERE), "oracle")


def test_reference_gpu_kernels_build_and_fail_cleanly():
    ref = O.reference_dir()
    if ref is None:
        pytest.skip("reference sources not present")
    subprocess.run(["make", "-s", "-C", ORACLE, "ref-gpu", f"REF={ref}"], check=True)
    lib = ctypes.CDLL(os.path.join(ORACLE, "_ref", "libdawn_ref_gpu.so"))
    for sym in ("ref_gpu_open", "ref_gpu_close", "ref_gpu_bfs", "ref_gpu_sssp"):
        assert hasattr(lib, sym), sym
    import torch
    if torch.cuda.is_available():
        return  # the device path is timed by oracle/time_ref_gpu.py
    lib.ref_gpu_open.restype = ctypes.c_void_p
    lib.ref_gpu_open.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int32, ctypes.c_int64, ctypes.c_int32]
    rp = np.array([0, 1, 2], np.int32)
    col = np.array([1, 0], np.int32)
    val = np.ones(2, np.float32)
    h = lib.ref_gpu_open(rp.ctypes.data, col.ctypes.data, val.ctypes.data, 2, 2, 1024)
    assert h is None
