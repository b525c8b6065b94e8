"""ctypes bindings of the C ABI in include/dawn_gb300.h (libdawn_gb300.so).

There is no fallback: the compute is the CUDA library.  A missing library
or a failing call raises :class:`DawnError` with the library's message.
"""

import ctypes
import os

import numpy as np

from . import LIB_DIR

OK, ERR_INVALID_ARG, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_UNSUPPORTED = 0, 1, 2, 3, 4, 5
W_NONE, W_I32, W_F32 = 0, 1, 2
GRAPH_SYMMETRIC, GRAPH_NO_VALIDATE = 1, 2
VARIANT_AUTO, VARIANT_PUSH, VARIANT_DO, VARIANT_BITSET, VARIANT_LEARNED = 0, 1, 2, 3, 4
INT32_MAX = np.iinfo(np.int32).max
FLT_MAX = np.float32(3.4028235e38)

LIB_PATH = os.path.join(LIB_DIR, "libdawn_gb300.so")

# Every symbol the header declares; tests check the library exports them.
EXPORTS = ("dawn_graph_create", "dawn_graph_create_device", "dawn_graph_destroy",
           "dawn_graph_set_stream", "dawn_graph_synchronize", "dawn_bfs", "dawn_bfs_device", "dawn_bfs_static",
           "dawn_sssp", "dawn_sssp_device", "dawn_closeness", "dawn_betweenness", "dawn_betweenness_device", "dawn_graph_set_option",
           "dawn_graph_get_option", "dawn_graph_set_selector", "dawn_autotune", "dawn_tune_cache_save",
           "dawn_tune_cache_load", "dawn_graph_set_parts", "dawn_multi_bfs", "dawn_multi_bfs_device",
           "dawn_multi_closeness", "dawn_trace_enable", "dawn_trace_read", "dawn_last_error", "dawn_version")
OPT_BITSET_WIDTH, OPT_PUSH_RATIO, OPT_FORCE_VARIANT, OPT_SELECTOR_MARGIN = 1, 2, 3, 4
OPT_PULL_SEGMENT, OPT_BLOCKS_PER_SM, OPT_AUTO_LEARNED, OPT_L2_PERSIST = 5, 6, 7, 8
OPT_SMALL_LEVELS = 9
TUNE_USE_CACHE = 1
SELECTOR_WEIGHTS = 1475


class Tuning(ctypes.Structure):
    _fields_ = [("bitset_width", ctypes.c_int32), ("push_ratio", ctypes.c_int32), ("pull_segment", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("learned", ctypes.c_int32), ("from_cache", ctypes.c_int32),
                ("ms", ctypes.c_float), ("default_ms", ctypes.c_float)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class DawnError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"dawn status {status}: {msg}")
        self.status = status


class Stats(ctypes.Structure):
    _fields_ = [("edges_traversed", ctypes.c_int64), ("levels", ctypes.c_int32),
                ("push_levels", ctypes.c_int32), ("pull_levels", ctypes.c_int32),
                ("batches", ctypes.c_int32), ("device_ms", ctypes.c_float)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}

    def __repr__(self):
        return "Stats(" + ", ".join(f"{k}={v}" for k, v in self.as_dict().items()) + ")"


class TraceRec(ctypes.Structure):
    _fields_ = [("kernel", ctypes.c_char * 24), ("run", ctypes.c_int32), ("level", ctypes.c_int32),
                ("mode", ctypes.c_int32), ("pad", ctypes.c_int32), ("frontier", ctypes.c_int64),
                ("frontier_edges", ctypes.c_int64), ("unvisited_edges", ctypes.c_int64),
                ("ms", ctypes.c_float), ("pad2", ctypes.c_float)]


_lib = None
_VP = ctypes.c_void_p
_I32P = ctypes.POINTER(ctypes.c_int32)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise DawnError(ERR_UNSUPPORTED, f"{LIB_PATH} missing: run __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        L.dawn_graph_create.argtypes = [_VP, _VP, _VP, ctypes.c_int, ctypes.c_int32, ctypes.c_int64,
                                        ctypes.c_uint32, _VP, ctypes.POINTER(_VP)]
        L.dawn_graph_create_device.argtypes = L.dawn_graph_create.argtypes
        L.dawn_graph_destroy.argtypes = [_VP]
        L.dawn_graph_set_stream.argtypes = [_VP, _VP]
        L.dawn_graph_synchronize.argtypes = [_VP]
        L.dawn_bfs.argtypes = [_VP, _VP, ctypes.c_int32, _VP, ctypes.c_int32, ctypes.POINTER(Stats)]
        L.dawn_bfs_device.argtypes = L.dawn_bfs.argtypes
        L.dawn_bfs_static.argtypes = [_VP, _VP, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, _VP,
                                      ctypes.c_uint32, _VP]
        L.dawn_sssp.argtypes = L.dawn_bfs.argtypes
        L.dawn_sssp_device.argtypes = L.dawn_bfs.argtypes
        L.dawn_closeness.argtypes = [_VP, _VP, ctypes.c_int32, ctypes.c_int32, _VP, _VP, _VP,
                                     ctypes.POINTER(Stats)]
        L.dawn_graph_set_option.argtypes = [_VP, ctypes.c_int32, ctypes.c_int64]
        L.dawn_graph_get_option.argtypes = [_VP, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]
        L.dawn_betweenness.argtypes = [_VP, _VP, ctypes.c_int32, _VP, ctypes.POINTER(Stats)]
        L.dawn_betweenness_device.argtypes = L.dawn_betweenness.argtypes
        L.dawn_graph_set_selector.argtypes = [_VP, _VP, ctypes.c_int32]
        L.dawn_autotune.argtypes = [_VP, _VP, ctypes.c_int32, ctypes.c_uint32, ctypes.POINTER(Tuning)]
        L.dawn_tune_cache_save.argtypes = [ctypes.c_char_p]
        L.dawn_tune_cache_load.argtypes = [ctypes.c_char_p]
        L.dawn_graph_set_parts.argtypes = [_VP, ctypes.c_int32, _VP]
        L.dawn_multi_bfs.argtypes = [_VP, _VP, _VP, _VP, ctypes.POINTER(Stats)]
        L.dawn_multi_bfs_device.argtypes = L.dawn_multi_bfs.argtypes
        L.dawn_multi_closeness.argtypes = [_VP, _VP, _VP, _VP, _VP, _VP, ctypes.POINTER(Stats)]
        L.dawn_trace_enable.argtypes = [_VP, ctypes.c_int32]
        L.dawn_trace_read.argtypes = [_VP, ctypes.POINTER(TraceRec), ctypes.c_int64,
                                      ctypes.POINTER(ctypes.c_int64)]
        for f in EXPORTS:
            getattr(L, f).restype = ctypes.c_int32
        L.dawn_last_error.restype = ctypes.c_char_p
        L.dawn_last_error.argtypes = []
        L.dawn_version.restype = ctypes.c_char_p
        L.dawn_version.argtypes = []
        _lib = L
    return _lib


def _check(rc):
    if rc != OK:
        raise DawnError(rc, lib().dawn_last_error().decode(errors="replace"))


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class Graph:
    """A CSR graph resident on the current CUDA device.

    ``g`` is any object with ``n``, ``row_ptr``, ``col`` and optional
    ``w_i32`` / ``w_f32`` / ``symmetric`` attributes (e.g. gen.CsrGraph).
    ``weights`` selects "i32", "f32" or None (unweighted).
    """

    def __init__(self, g=None, weights=None, symmetric=None, stream=None, validate=True, raw=None):
        if raw is not None:
            self._init_raw(**raw)
            return
        self.n = int(g.n)
        self._rp = np.ascontiguousarray(g.row_ptr, np.int32)
        self._col = np.ascontiguousarray(g.col, np.int32)
        self.m = int(self._col.shape[0])
        self.wtype = {None: W_NONE, "i32": W_I32, "f32": W_F32}[weights]
        self._val = None
        if self.wtype == W_I32:
            self._val = np.ascontiguousarray(g.w_i32, np.int32)
        elif self.wtype == W_F32:
            self._val = np.ascontiguousarray(g.w_f32, np.float32)
        sym = bool(getattr(g, "symmetric", False)) if symmetric is None else bool(symmetric)
        flags = (GRAPH_SYMMETRIC if sym else 0) | (0 if validate else GRAPH_NO_VALIDATE)
        h = ctypes.c_void_p()
        _check(lib().dawn_graph_create(_ptr(self._rp), _ptr(self._col), _ptr(self._val), self.wtype,
                                       self.n, self.m, flags, ctypes.c_void_p(stream or 0),
                                       ctypes.byref(h)))
        self.handle = h
        self.degrees = np.diff(self._rp.astype(np.int64))

    def _init_raw(self, n, m, row_ptr, col, val=0, wtype=W_NONE, symmetric=False, stream=None,
                  validate=True, device=False):
        """Create from raw pointers (host, or device when device=True)."""
        self.n, self.m, self.wtype = int(n), int(m), wtype
        self._rp = self._col = self._val = None
        flags = (GRAPH_SYMMETRIC if symmetric else 0) | (0 if validate else GRAPH_NO_VALIDATE)
        h = ctypes.c_void_p()
        fn = lib().dawn_graph_create_device if device else lib().dawn_graph_create
        _check(fn(ctypes.c_void_p(row_ptr), ctypes.c_void_p(col), ctypes.c_void_p(val or 0), wtype, self.n,
                  self.m, flags, ctypes.c_void_p(stream or 0), ctypes.byref(h)))
        self.handle = h
        self.degrees = None

    def bfs_host_ptr(self, sources, dist_ptr, variant=VARIANT_AUTO):
        """dawn_bfs into a caller host buffer (e.g. pinned memory)."""
        s = np.ascontiguousarray(sources, np.int32)
        st = Stats()
        _check(lib().dawn_bfs(self.handle, _ptr(s), len(s), ctypes.c_void_p(dist_ptr), variant,
                              ctypes.byref(st)))
        return st

    # -- lifetime --
    def close(self):
        if self.handle:
            _check(lib().dawn_graph_destroy(self.handle))
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        _check(lib().dawn_graph_set_stream(self.handle, ctypes.c_void_p(stream or 0)))

    def synchronize(self):
        _check(lib().dawn_graph_synchronize(self.handle))

    def set_option(self, option, value):
        _check(lib().dawn_graph_set_option(self.handle, option, int(value)))

    def get_option(self, option):
        v = ctypes.c_int64()
        _check(lib().dawn_graph_get_option(self.handle, option, ctypes.byref(v)))
        return v.value

    def autotune(self, sources, use_cache=False):
        """dawn_autotune: measure and set this handle's speed settings."""
        s = np.ascontiguousarray(sources, np.int32)
        t = Tuning()
        _check(lib().dawn_autotune(self.handle, _ptr(s), len(s), TUNE_USE_CACHE if use_cache else 0,
                                   ctypes.byref(t)))
        return t.as_dict()

    def betweenness(self, sources=None):
        """dawn_betweenness over `sources` (default: every vertex, the
        reference's BC_CPU::Betweenness_Centrality)."""
        s = np.arange(self.n, dtype=np.int32) if sources is None else np.ascontiguousarray(sources, np.int32)
        bc = np.empty(self.n, np.float64)
        st = Stats()
        _check(lib().dawn_betweenness(self.handle, _ptr(s), len(s), _ptr(bc), ctypes.byref(st)))
        return bc, st

    def set_selector(self, weights):
        """dawn_graph_set_selector: load MLP weights (1475 floats) or None."""
        if weights is None:
            _check(lib().dawn_graph_set_selector(self.handle, None, 0))
            return
        w = np.ascontiguousarray(weights, np.float32)
        _check(lib().dawn_graph_set_selector(self.handle, _ptr(w), int(w.size)))

    def bfs_stats(self, sources, variant=VARIANT_AUTO):
        """dawn_bfs with dist = NULL: the traversal runs, only statistics return."""
        s = np.ascontiguousarray(sources, np.int32)
        st = Stats()
        _check(lib().dawn_bfs(self.handle, _ptr(s), len(s), None, variant, ctypes.byref(st)))
        return st

    def set_parts(self, offsets):
        """dawn_graph_set_parts: the graph is the disjoint union of the
        vertex ranges [offsets[p], offsets[p+1])."""
        self._parts = np.ascontiguousarray(offsets, np.int32)
        _check(lib().dawn_graph_set_parts(self.handle, len(self._parts) - 1, _ptr(self._parts)))

    def _multi_args(self, sources_per_part):
        so = np.zeros(len(self._parts), np.int32)
        so[1:] = np.cumsum([len(s) for s in sources_per_part])
        src = (np.concatenate([np.asarray(s, np.int32) for s in sources_per_part]) if len(sources_per_part)
               else np.zeros(0, np.int32))
        return so, np.ascontiguousarray(src, np.int32)

    def multi_out_size(self, sources_per_part):
        sizes = np.diff(self._parts.astype(np.int64))
        return int(sum(len(s) * int(sizes[p]) for p, s in enumerate(sources_per_part)))

    def multi_bfs(self, sources_per_part, out=None):
        """dawn_multi_bfs: returns (list of per-part (sources x n_p) blocks, stats)."""
        so, src = self._multi_args(sources_per_part)
        d = out if out is not None else np.empty(self.multi_out_size(sources_per_part), np.int32)
        st = Stats()
        _check(lib().dawn_multi_bfs(self.handle, _ptr(so), _ptr(src), _ptr(d), ctypes.byref(st)))
        blocks, o = [], 0
        sizes = np.diff(self._parts.astype(np.int64))
        for p, s in enumerate(sources_per_part):
            k, npart = len(s), int(sizes[p])
            blocks.append(d[o:o + k * npart].reshape(k, npart))
            o += k * npart
        return blocks, st

    def multi_bfs_ptr(self, sources_per_part, dist_ptr, device=False, stats=True):
        """dawn_multi_bfs (host pointer) or dawn_multi_bfs_device into a raw buffer."""
        so, src = self._multi_args(sources_per_part)
        st = Stats() if stats else None
        fn = lib().dawn_multi_bfs_device if device else lib().dawn_multi_bfs
        _check(fn(self.handle, _ptr(so), _ptr(src), ctypes.c_void_p(dist_ptr),
                  ctypes.byref(st) if st is not None else None))
        return st

    def multi_closeness(self, sources_per_part):
        so, src = self._multi_args(sources_per_part)
        cc = np.empty(len(src), np.float64)
        ds = np.empty(len(src), np.float64)
        rc = np.empty(len(src), np.int64)
        st = Stats()
        _check(lib().dawn_multi_closeness(self.handle, _ptr(so), _ptr(src), _ptr(cc), _ptr(ds), _ptr(rc),
                                          ctypes.byref(st)))
        return cc, ds, rc, st

    def trace(self, enable=True):
        _check(lib().dawn_trace_enable(self.handle, int(enable)))

    def trace_read(self):
        """All pending per-level records as a list of dicts."""
        out = []
        buf = (TraceRec * 4096)()
        while True:
            cnt = ctypes.c_int64()
            _check(lib().dawn_trace_read(self.handle, buf, 4096, ctypes.byref(cnt)))
            for r in buf[:cnt.value]:
                out.append({"kernel": r.kernel.decode(), "run": r.run, "level": r.level, "mode": r.mode,
                            "frontier": r.frontier, "frontier_edges": r.frontier_edges,
                            "unvisited_edges": r.unvisited_edges, "ms": r.ms, "pad": r.pad})
            if cnt.value < 4096:
                return out

    # -- traversals (host buffers) --
    def bfs(self, sources, variant=VARIANT_AUTO, out=None):
        s = np.ascontiguousarray(sources, np.int32)
        d = out if out is not None else np.empty((len(s), self.n), np.int32)
        st = Stats()
        _check(lib().dawn_bfs(self.handle, _ptr(s), len(s), _ptr(d), variant, ctypes.byref(st)))
        return d, st

    def sssp(self, sources, out=None, variant=VARIANT_AUTO):
        """Weighted distances; AUTO batches 64 sources per traversal, DO/PUSH
        run the single-source kernels."""
        s = np.ascontiguousarray(sources, np.int32)
        dt = np.float32 if self.wtype == W_F32 else np.int32
        d = out if out is not None else np.empty((len(s), self.n), dt)
        st = Stats()
        _check(lib().dawn_sssp(self.handle, _ptr(s), len(s), _ptr(d), variant, ctypes.byref(st)))
        return d, st

    def closeness(self, sources, weighted=False, with_stats=False):
        s = np.ascontiguousarray(sources, np.int32)
        cc = np.empty(len(s), np.float64)
        sums = np.empty(len(s), np.float64)
        reached = np.empty(len(s), np.int64)
        st = Stats()
        _check(lib().dawn_closeness(self.handle, _ptr(s), len(s), int(weighted), _ptr(cc), _ptr(sums),
                                    _ptr(reached), ctypes.byref(st)))
        return (cc, sums, reached, st) if with_stats else (cc, sums, reached)

    # -- traversals (device buffers, e.g. torch tensors' data_ptr()) --
    def bfs_device(self, sources, d_dist, variant=VARIANT_AUTO, stats=True):
        s = np.ascontiguousarray(sources, np.int32)
        st = Stats() if stats else None
        _check(lib().dawn_bfs_device(self.handle, _ptr(s), len(s), ctypes.c_void_p(d_dist), variant,
                                     ctypes.byref(st) if st is not None else None))
        return st

    def sssp_device(self, sources, d_dist, stats=True, variant=VARIANT_AUTO):
        s = np.ascontiguousarray(sources, np.int32)
        st = Stats() if stats else None
        _check(lib().dawn_sssp_device(self.handle, _ptr(s), len(s), ctypes.c_void_p(d_dist), variant,
                                      ctypes.byref(st) if st is not None else None))
        return st


STATIC_MAX_VERTICES, STATIC_MAX_EDGES = 1 << 20, 1 << 24
PART_MAX_VERTICES = 1 << 18


def bfs_static(row_ptr, col, n, m, source, dist, flags=0, stream=None):
    """dawn_bfs_static: hop distances from one source into `dist`, with the
    CSR and `dist` given as device addresses (ints) of the current device.
    Allocates nothing; graphs beyond STATIC_MAX_VERTICES / STATIC_MAX_EDGES
    raise DawnError.  Calls that overlap on one device race."""
    _check(lib().dawn_bfs_static(ctypes.c_void_p(row_ptr), ctypes.c_void_p(col), n, m, source,
                                 ctypes.c_void_p(dist), flags, ctypes.c_void_p(stream)))


def tune_cache_save(path):
    _check(lib().dawn_tune_cache_save(os.fsencode(path)))


def tune_cache_load(path):
    _check(lib().dawn_tune_cache_load(os.fsencode(path)))


def version():
    return lib().dawn_version().decode()
