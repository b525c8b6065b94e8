"""ORACLE — test infrastructure only.

ctypes bindings for the C restatement (``lib/liboracle.so``) and, when it was
built here, for the reference compiled from its own sources
(``_ref/libdawn_ref.so``).  Only tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "lib", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libdawn_ref.so")
REF_BIN = os.path.join(HERE, "_ref", "bin")

_I = ctypes.POINTER(ctypes.c_int32)
_F = ctypes.POINTER(ctypes.c_float)
_U8 = ctypes.POINTER(ctypes.c_uint8)


# The reference's source tree: $DAWN_REFERENCE_DIR, by default the read-only
# checkout at /root/reference.  Machines without it (the GPU hosts) use the
# install copy that stage_reference() leaves, untracked, under baseline/_ref/.
REF_DEFAULT = "/root/reference"
STAGED = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "GAL-DAWN")
STAGE_PARTS = ("src", "include", "algorithm", "LICENSE")


def _has_src(d):
    return bool(d) and os.path.isdir(os.path.join(d, "src", "algorithm", "cpu"))


def reference_dir():
    """The reference sources to compile from, or None."""
    d = os.environ.get("DAWN_REFERENCE_DIR", REF_DEFAULT)
    if _has_src(d):
        return d
    return STAGED if _has_src(STAGED) else None


def stage_reference(ref_dir):
    """Install copy of the unmodified reference sources under baseline/_ref/
    (git-ignored, carried to GPU hosts with the working tree), so the
    reference's own CPU path can be compiled on a machine that has no
    checkout of it.  Nothing under it is ever edited."""
    import shutil
    if os.path.realpath(ref_dir) == os.path.realpath(STAGED):
        return
    os.makedirs(STAGED, exist_ok=True)
    for part in STAGE_PARTS:
        src, dst = os.path.join(ref_dir, part), os.path.join(STAGED, part)
        if os.path.isdir(src):
            shutil.copytree(src, dst, dirs_exist_ok=True)
        elif os.path.exists(src):
            shutil.copy2(src, dst)


def build(ref_dir=None, with_ref=None):
    """Compile the restatement, and the reference wherever its sources are
    found (the checkout, or the staged install copy)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref_dir = ref_dir or reference_dir()
    if with_ref is None:
        with_ref = _has_src(ref_dir)
    if with_ref:
        stage_reference(ref_dir)
        subprocess.run(["make", "-s", "-C", HERE, "-j8", "ref", f"REF={ref_dir}"], check=True)


def _ip(a):
    return a.ctypes.data_as(_I)


def _fp(a):
    return a.ctypes.data_as(_F)


_port = None
_ref = None


def port():
    global _port
    if _port is None:
        if not os.path.exists(LIB):
            build(with_ref=False)
        L = ctypes.CDLL(LIB)
        L.oracle_bfs_queue.argtypes = [_I, _I, ctypes.c_int32, ctypes.c_int32, _I]
        L.oracle_bfs_queue.restype = ctypes.c_int64
        L.oracle_bfs_bitmap.argtypes = [_I, _I, ctypes.c_int32, ctypes.c_int32, _I]
        L.oracle_bfs_bitmap.restype = None
        L.oracle_sssp.argtypes = [_I, _I, _F, ctypes.c_int32, ctypes.c_int32, _F]
        L.oracle_sssp.restype = None
        L.oracle_mssp.argtypes = [_I, _I, ctypes.c_int32, _I, ctypes.c_int32,
                                  ctypes.c_int32, _I, _U8]
        L.oracle_bc.argtypes = [_I, _I, ctypes.c_int32, _I, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_bc.restype = None
        L.oracle_mssp.restype = ctypes.c_int64
        L.oracle_msssp.argtypes = [_I, _I, _F, ctypes.c_int32, _I, ctypes.c_int32,
                                   ctypes.c_int32, _F]
        L.oracle_msssp.restype = None
        L.oracle_closeness_hops.argtypes = [_I, ctypes.c_int32, ctypes.c_int32]
        L.oracle_closeness_hops.restype = ctypes.c_double
        L.oracle_closeness_weighted.argtypes = [_F, ctypes.c_int32, ctypes.c_int32]
        L.oracle_closeness_weighted.restype = ctypes.c_double
        L.oracle_closeness_ref_int.argtypes = [_I, ctypes.c_int32, ctypes.c_int32]
        L.oracle_closeness_ref_int.restype = ctypes.c_float
        L.oracle_num_threads.restype = ctypes.c_int
        _port = L
    return _port


def ref_available() -> bool:
    if not os.path.exists(REF_LIB):
        return False
    try:
        ref()
        return True
    except OSError:
        return False


def ref():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_LIB)
        L.ref_bfs_kernel.argtypes = [_I, _I, ctypes.c_int32, ctypes.c_int32, _I]
        L.ref_bc.argtypes = [_I, _I, ctypes.c_int32, _F]
        L.ref_bc.restype = None
        L.ref_bfs_bitmap.argtypes = [_I, _I, ctypes.c_int32, ctypes.c_int32, _I]
        L.ref_sssp.argtypes = [_I, _I, _F, ctypes.c_int32, ctypes.c_int32, _F]
        L.ref_cc.argtypes = [_I, _I, _F, ctypes.c_int32, ctypes.c_int32]
        L.ref_cc.restype = ctypes.c_float
        L.ref_mssp_run.argtypes = [_I, _I, _F, ctypes.c_int32, ctypes.c_int64, _I,
                                   ctypes.c_int32, ctypes.c_int32, _I, _F]
        L.ref_mssp_run.restype = ctypes.c_float
        _ref = L
    return _ref


def _csr(g):
    return (np.ascontiguousarray(g.row_ptr, np.int32), np.ascontiguousarray(g.col, np.int32))


# --- restatement -----------------------------------------------------------

def bfs_queue(g, source):
    """Reference-encoded hop distances (0 = unvisited / source) and TEPS edges."""
    rp, col = _csr(g)
    d = np.zeros(g.n, np.int32)
    e = port().oracle_bfs_queue(_ip(rp), _ip(col), g.n, int(source), _ip(d))
    return d, int(e)


def bfs_bitmap(g, source):
    rp, col = _csr(g)
    d = np.zeros(g.n, np.int32)
    port().oracle_bfs_bitmap(_ip(rp), _ip(col), g.n, int(source), _ip(d))
    return d


def sssp(g, source, val=None):
    rp, col = _csr(g)
    v = np.ascontiguousarray(g.w_f32 if val is None else val, np.float32)
    d = np.zeros(g.n, np.float32)
    port().oracle_sssp(_ip(rp), _ip(col), _fp(v), g.n, int(source), _fp(d))
    return d


def mssp(g, sources, threads=0, want_dist=True):
    rp, col = _csr(g)
    s = np.ascontiguousarray(sources, np.int32)
    d = np.zeros((len(s), g.n), np.int32) if want_dist else None
    skipped = np.zeros(len(s), np.uint8)
    e = port().oracle_mssp(_ip(rp), _ip(col), g.n, _ip(s), len(s), threads,
                           _ip(d) if d is not None else None,
                           skipped.ctypes.data_as(_U8))
    return d, int(e), skipped.astype(bool)


def msssp(g, sources, threads=0, val=None):
    rp, col = _csr(g)
    v = np.ascontiguousarray(g.w_f32 if val is None else val, np.float32)
    s = np.ascontiguousarray(sources, np.int32)
    d = np.zeros((len(s), g.n), np.float32)
    port().oracle_msssp(_ip(rp), _ip(col), _fp(v), g.n, _ip(s), len(s), threads, _fp(d))
    return d


def closeness_hops(dist_ref_row, source):
    d = np.ascontiguousarray(dist_ref_row, np.int32)
    return port().oracle_closeness_hops(_ip(d), d.shape[0], int(source))


def closeness_weighted(dist_row, source):
    d = np.ascontiguousarray(dist_row, np.float32)
    return port().oracle_closeness_weighted(_fp(d), d.shape[0], int(source))


def closeness_ref_int(dist_ref_row, source):
    d = np.ascontiguousarray(dist_ref_row, np.int32)
    return port().oracle_closeness_ref_int(_ip(d), d.shape[0], int(source))


def bc(g, sources=None, exact_ref_order=False):
    """BCDAWN betweenness summed over `sources` (default: every vertex):
    float64 restatement, or with exact_ref_order the reference's float32
    arithmetic in its order."""
    rp, col = _csr(g)
    s = np.arange(g.n, dtype=np.int32) if sources is None else np.ascontiguousarray(sources, np.int32)
    if exact_ref_order:
        out = np.zeros(g.n, np.float32)
        port().oracle_bc(_ip(rp), _ip(col), g.n, _ip(s), len(s), None, out.ctypes.data)
    else:
        out = np.zeros(g.n, np.float64)
        port().oracle_bc(_ip(rp), _ip(col), g.n, _ip(s), len(s), out.ctypes.data, None)
    return out


def num_threads():
    return port().oracle_num_threads()


# --- encodings ---------------------------------------------------------------

def hops_ref_to_api(dist_ref, sources):
    """Reference encoding (0 = unvisited, source 0) -> C-ABI encoding (-1 unreachable)."""
    d = np.array(dist_ref, np.int32, copy=True)
    d2 = d.reshape(-1, d.shape[-1])
    src = np.atleast_1d(np.asarray(sources))
    for i, s in enumerate(src):
        row = d2[i]
        row[row == 0] = -1
        row[int(s) % row.shape[0]] = 0
    return d2.reshape(d.shape)


# --- the reference itself (built here only) ----------------------------------

def ref_bfs_kernel(g, source):
    rp, col = _csr(g)
    d = np.zeros(g.n, np.int32)
    ref().ref_bfs_kernel(_ip(rp), _ip(col), g.n, int(source), _ip(d))
    return d


def ref_bfs_bitmap(g, source):
    rp, col = _csr(g)
    d = np.zeros(g.n, np.int32)
    ref().ref_bfs_bitmap(_ip(rp), _ip(col), g.n, int(source), _ip(d))
    return d


def ref_sssp(g, source, val=None):
    rp, col = _csr(g)
    v = np.ascontiguousarray(g.w_f32 if val is None else val, np.float32)
    d = np.zeros(g.n, np.float32)
    ref().ref_sssp(_ip(rp), _ip(col), _fp(v), g.n, int(source), _fp(d))
    return d


def ref_cc(g, source, weighted=False):
    rp, col = _csr(g)
    v = np.ascontiguousarray(g.w_f32, np.float32) if weighted else None
    return ref().ref_cc(_ip(rp), _ip(col), _fp(v) if v is not None else None, g.n, int(source))


def ref_mssp(g, sources, want_dist=True):
    rp, col = _csr(g)
    s = np.ascontiguousarray(sources, np.int32)
    d = np.zeros((len(s), g.n), np.int32) if want_dist else None
    t = ref().ref_mssp_run(_ip(rp), _ip(col), None, g.n, g.m, _ip(s), len(s), 0,
                           _ip(d) if d is not None else None, None)
    return d, t


def ref_bc(g):
    """The reference's BC_CPU::Betweenness_Centrality (every vertex a source)."""
    rp, col = _csr(g)
    out = np.zeros(g.n, np.float32)
    ref().ref_bc(_ip(rp), _ip(col), g.n, _fp(out))
    return out
