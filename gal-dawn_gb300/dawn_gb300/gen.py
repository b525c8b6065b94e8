"""Seeded graph generators (libdawn_gen.so) returning numpy CSR graphs.

The generators are deterministic across machines and thread counts; see
``csrc/gen.cpp``.  The workload presets match the benchmark configurations:
directed Erdos-Renyi, symmetrised RMAT, 2D grid and random-geometric kNN.
"""

import ctypes
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import LIB_DIR

SYMMETRIC, DEDUP, NO_SELF, WEIGHTS, PERMUTE = 1, 2, 4, 8, 16


class _Csr(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("m", ctypes.c_int64),
                ("row_ptr", ctypes.POINTER(ctypes.c_int32)),
                ("col", ctypes.POINTER(ctypes.c_int32)),
                ("w_i32", ctypes.POINTER(ctypes.c_int32)),
                ("w_f32", ctypes.POINTER(ctypes.c_float))]


@dataclass
class CsrGraph:
    """Host CSR graph: int32 row_ptr[n+1], int32 col[m], optional weights."""
    n: int
    row_ptr: np.ndarray
    col: np.ndarray
    w_i32: Optional[np.ndarray] = None
    w_f32: Optional[np.ndarray] = None
    symmetric: bool = False
    name: str = ""

    @property
    def m(self) -> int:
        return int(self.col.shape[0])

    def degrees(self) -> np.ndarray:
        return np.diff(self.row_ptr.astype(np.int64))


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(LIB_DIR, "libdawn_gen.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build()")
        L = ctypes.CDLL(path)
        P = ctypes.POINTER(_Csr)
        L.dawn_gen_rmat.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                    ctypes.c_int, P]
        L.dawn_gen_er.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64,
                                  ctypes.c_int, P]
        L.dawn_gen_grid.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64,
                                    ctypes.c_int, P]
        L.dawn_gen_knn.argtypes = [ctypes.c_int32, ctypes.c_int, ctypes.c_uint64,
                                   ctypes.c_int, P]
        L.dawn_gen_sources.argtypes = [P, ctypes.c_int32, ctypes.c_uint64, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int32)]
        L.dawn_write_mtx.argtypes = [P, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
        L.dawn_csr_free.argtypes = [P]
        for f in ("dawn_gen_rmat", "dawn_gen_er", "dawn_gen_grid", "dawn_gen_knn",
                  "dawn_gen_sources", "dawn_write_mtx"):
            getattr(L, f).restype = ctypes.c_int
        L.dawn_csr_free.restype = None
        _lib = L
    return _lib


def _take(c: _Csr, flags: int, name: str) -> CsrGraph:
    n, m = int(c.n), int(c.m)
    rp = np.ctypeslib.as_array(c.row_ptr, shape=(n + 1,)).copy()
    col = np.ctypeslib.as_array(c.col, shape=(max(m, 1),))[:m].copy()
    wi = wf = None
    if flags & WEIGHTS:
        wi = np.ctypeslib.as_array(c.w_i32, shape=(max(m, 1),))[:m].copy()
        wf = np.ctypeslib.as_array(c.w_f32, shape=(max(m, 1),))[:m].copy()
    lib().dawn_csr_free(ctypes.byref(c))
    return CsrGraph(n, rp, col, wi, wf, bool(flags & SYMMETRIC), name)


def _check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"{what} failed with status {rc}")


def rmat(scale: int, edgefactor: int = 16, a=0.57, b=0.19, c=0.19, seed=1,
         weights=False, symmetric=True, permute=True) -> CsrGraph:
    flags = DEDUP | NO_SELF | (SYMMETRIC if symmetric else 0) | \
        (WEIGHTS if weights else 0) | (PERMUTE if permute else 0)
    out = _Csr()
    _check(lib().dawn_gen_rmat(scale, edgefactor, a, b, c, seed, flags,
                               ctypes.byref(out)), "dawn_gen_rmat")
    return _take(out, flags, f"rmat{scale}")


def erdos_renyi(n: int, nedges: int, seed=1, weights=False,
                symmetric=False) -> CsrGraph:
    flags = DEDUP | NO_SELF | (SYMMETRIC if symmetric else 0) | \
        (WEIGHTS if weights else 0)
    out = _Csr()
    _check(lib().dawn_gen_er(n, nedges, seed, flags, ctypes.byref(out)), "dawn_gen_er")
    return _take(out, flags, f"er{n}")


def grid(rows: int, cols: int, seed=1, weights=False) -> CsrGraph:
    flags = DEDUP | NO_SELF | SYMMETRIC | (WEIGHTS if weights else 0)
    out = _Csr()
    _check(lib().dawn_gen_grid(rows, cols, seed, flags, ctypes.byref(out)), "dawn_gen_grid")
    return _take(out, flags, f"grid{rows}x{cols}")


def knn(npts: int, k: int = 8, seed=1, weights=False) -> CsrGraph:
    flags = DEDUP | NO_SELF | SYMMETRIC | (WEIGHTS if weights else 0)
    out = _Csr()
    _check(lib().dawn_gen_knn(npts, k, seed, flags, ctypes.byref(out)), "dawn_gen_knn")
    return _take(out, flags, f"knn{npts}")


def _as_csr_struct(g: CsrGraph):
    c = _Csr()
    c.n = g.n
    c.m = g.m
    keep = [np.ascontiguousarray(g.row_ptr, np.int32), np.ascontiguousarray(g.col, np.int32)]
    c.row_ptr = keep[0].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    c.col = keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    if g.w_i32 is not None:
        keep.append(np.ascontiguousarray(g.w_i32, np.int32))
        c.w_i32 = keep[-1].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    return c, keep


def sources(g: CsrGraph, nsrc: int, seed=7, from_lcc=True) -> np.ndarray:
    c, keep = _as_csr_struct(g)
    out = np.zeros(nsrc, np.int32)
    _check(lib().dawn_gen_sources(ctypes.byref(c), nsrc, seed, int(from_lcc),
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))),
           "dawn_gen_sources")
    return out


def write_mtx(g: CsrGraph, path: str, weighted=False):
    c, keep = _as_csr_struct(g)
    _check(lib().dawn_write_mtx(ctypes.byref(c), path.encode(), int(g.symmetric),
                                int(weighted)), "dawn_write_mtx")


def disjoint_union(graphs):
    """One CSR holding ``graphs`` side by side: vertex v of part p becomes
    offsets[p] + v.  Returns (CsrGraph, int32 offsets[nparts + 1])."""
    ns = np.array([g.n for g in graphs], np.int64)
    ms = np.array([g.m for g in graphs], np.int64)
    voff = np.concatenate([[0], np.cumsum(ns)])
    eoff = np.concatenate([[0], np.cumsum(ms)])
    if voff[-1] >= 2**31 or eoff[-1] >= 2**31:
        raise ValueError("the union exceeds int32 vertex or edge ids")
    rp = np.empty(int(voff[-1]) + 1, np.int32)
    col = np.empty(int(eoff[-1]), np.int32)
    weighted = all(g.w_i32 is not None for g in graphs)
    wi = np.empty(int(eoff[-1]), np.int32) if weighted else None
    wf = np.empty(int(eoff[-1]), np.float32) if weighted else None
    for p, g in enumerate(graphs):
        rp[voff[p]:voff[p + 1]] = g.row_ptr[:-1] + eoff[p]
        col[eoff[p]:eoff[p + 1]] = g.col + voff[p]
        if weighted:
            wi[eoff[p]:eoff[p + 1]] = g.w_i32
            wf[eoff[p]:eoff[p + 1]] = g.w_f32
    rp[-1] = eoff[-1]
    u = CsrGraph(int(voff[-1]), rp, col, wi, wf, symmetric=all(g.symmetric for g in graphs),
                 name=f"union{len(graphs)}")
    return u, voff.astype(np.int32)


def er_family(ngraphs=512, nmin=1024, nmax=65536, dmin=4, dmax=32, smin=8, smax=64, seed=1):
    """Independent directed Erdos-Renyi graphs with n uniform in [nmin, nmax],
    average out-degree uniform in [dmin, dmax] and smin..smax sources each
    (drawn uniformly, with the generator's seeds derived from ``seed``).
    Returns (graphs, list of int32 source arrays)."""
    rng = np.random.default_rng(seed)
    graphs, srcs = [], []
    for i in range(ngraphs):
        n = int(rng.integers(nmin, nmax + 1))
        d = float(rng.uniform(dmin, dmax))
        g = erdos_renyi(n, int(round(n * d)), seed=int(rng.integers(1, 2**62)))
        graphs.append(g)
        k = int(rng.integers(smin, smax + 1))
        srcs.append(rng.integers(0, n, size=k).astype(np.int32))
    return graphs, srcs
