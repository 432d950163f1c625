"""ctypes wrapper of the oracle (oracle/gx_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the correctness reference, and by bench.py's CPU-baseline leg.  The product path never
imports it.  Pinned against the reference's own outputs in tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libgxoracle.so"

PAGERANK_REF, PAGERANK_STD, SSSP, CC, INDEGREE, PAGERANK_REF64 = range(6)
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)
        L = C.CDLL(str(LIB))
        P, I32 = C.c_void_p, C.c_int32
        L.gxo_run.restype = C.c_int
        L.gxo_run.argtypes = [C.c_int, I32, I32, P, P, P, P, P, I32, C.c_double, I32, C.c_double, C.c_int,
                              P, P, P, P, P]
        L.gxo_triangles.restype = C.c_uint64
        L.gxo_triangles.argtypes = [I32, P, P, C.c_int]
        L.gxo_ppr.restype = C.c_int
        L.gxo_ppr.argtypes = [I32, P, P, P, I32, P, I32, C.c_double, C.c_int, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def run(app, V, P, bounds, off, col, outdeg, max_iter, weights=None, damping=0.85, source=1, tolerance=0.0,
        threads=0, init=None):
    """GraphPS<T>::run with the chosen vertex program.  Returns
    (values, changed_per_step, ms_per_step)."""
    dt = {PAGERANK_REF: np.float32, PAGERANK_STD: np.float64, PAGERANK_REF64: np.float64,
          SSSP: np.uint32 if weights is not None else np.int32, CC: np.int32, INDEGREE: np.int32}[app]
    out = np.empty(V, dt)
    changed = np.zeros(max(max_iter, 1), np.int64)
    ms = np.zeros(max(max_iter, 1), np.float64)
    iters = C.c_int32(0)
    bounds = np.ascontiguousarray(bounds, np.int32)
    off = np.ascontiguousarray(off, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    outdeg = np.ascontiguousarray(outdeg, np.int32)
    w = None if weights is None else np.ascontiguousarray(weights, np.uint32)
    ini = None if init is None else np.ascontiguousarray(init, dt)
    rc = lib().gxo_run(app, V, P, _p(bounds), _p(off), _p(col), _p(outdeg), _p(w), max_iter, damping, source,
                       tolerance, threads, _p(ini), _p(out), _p(changed), _p(ms), C.byref(iters))
    if rc != 0:
        raise RuntimeError(f"gxo_run failed with {rc}")
    n = iters.value
    return out, changed[:n].copy(), ms[:n].copy()


def triangles(V, off, col, threads=0) -> int:
    off = np.ascontiguousarray(off, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    return int(lib().gxo_triangles(V, _p(off), _p(col), threads))


def ppr(V, off, col, outdeg, sources, iters, restart=0.15, threads=0):
    sources = np.ascontiguousarray(sources, np.int32)
    k = len(sources)
    out = np.empty((V, k), np.float64)
    rc = lib().gxo_ppr(V, _p(np.ascontiguousarray(off, np.int64)), _p(np.ascontiguousarray(col, np.int32)),
                       _p(np.ascontiguousarray(outdeg, np.int32)), k, _p(sources), iters, restart, threads, _p(out))
    if rc != 0:
        raise RuntimeError("gxo_ppr failed")
    return out
