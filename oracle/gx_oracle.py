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
        D, I64, U64 = C.c_double, C.c_int64, C.c_uint64
        L.gxo_rmat_csc.restype = C.c_int
        L.gxo_rmat_csc.argtypes = [I32, I64, D, D, D, U64, I32, I32, I32, C.c_int, P, P, P]
        L.gxo_partition_bounds.restype = C.c_int
        L.gxo_partition_bounds.argtypes = [I32, P, I32, P]
        L.gxo_out_degree.restype = C.c_int
        L.gxo_out_degree.argtypes = [I32, P, P, C.c_int, P]
        L.gxo_edge_weights.restype = C.c_int
        L.gxo_edge_weights.argtypes = [U64, I32, P, P, C.c_int, P]
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


class Graph:
    """A graph in the shard layout the engine takes: bounds[P+1], off[V+1],
    col[E], outdeg[V] (and weights[E] when asked for)."""

    def __init__(self, V, off, col, outdeg, P, bounds, weights=None):
        self.V, self.off, self.col, self.outdeg, self.P, self.bounds = V, off, col, outdeg, P, bounds
        self.weights = weights

    @property
    def E(self) -> int:
        return int(self.off[-1])


def rmat_graph(scale, edge_factor, seed, P=1, symmetric=False, a=0.57, b=0.19, c=0.19, weight_seed=None,
               threads=0) -> Graph:
    """The library's seeded R-MAT graph (self-loops and duplicates removed,
    optionally symmetrised) built by the oracle alone, with P edge-balanced
    shards and, when weight_seed is given, SSSP weights."""
    V = 1 << scale
    n = edge_factor * V
    off = np.empty(V + 1, np.int64)
    col = np.empty(max(2 * n if symmetric else n, 1), np.int32)
    nout = C.c_int64(0)
    rc = lib().gxo_rmat_csc(scale, n, a, b, c, seed & 0xFFFFFFFFFFFFFFFF, 1, 1, int(symmetric), threads, _p(off),
                            _p(col), C.byref(nout))
    if rc != 0:
        raise RuntimeError("gxo_rmat_csc failed")
    col = col[:nout.value].copy()
    outdeg = np.empty(V, np.int32)
    bounds = np.empty(P + 1, np.int32)
    if lib().gxo_out_degree(V, _p(off), _p(col), threads, _p(outdeg)) != 0 or \
            lib().gxo_partition_bounds(V, _p(off), P, _p(bounds)) != 0:
        raise RuntimeError("oracle graph construction failed")
    g = Graph(V, off, col, outdeg, P, bounds)
    if weight_seed is not None:
        w = np.empty(max(g.E, 1), np.uint32)
        if lib().gxo_edge_weights(weight_seed & 0xFFFFFFFFFFFFFFFF, V, _p(off), _p(col), threads, _p(w)) != 0:
            raise RuntimeError("gxo_edge_weights failed")
        g.weights = w[:g.E]
    return g


def write_shards(g: Graph, directory: str) -> str:
    """Writes the graph as the reference's shard directory: {p}.edge.npy =
    int32 [E_p, len(indices), len(indptr), start, end, indices..., indptr...]
    for each destination range (GraphMP/tools/format_spark.py:137-157, read
    by GraphMP/system/Comp.h:33-42), vertexout.npy and vertexin.npy (int32[V],
    GraphMP/system/GraphPS.h:162-169)."""
    import os
    d = str(directory)
    if not d.endswith("/"):
        d += "/"
    os.makedirs(d, exist_ok=True)
    for p in range(g.P):
        s, e = int(g.bounds[p]), int(g.bounds[p + 1])
        lo, hi = int(g.off[s]), int(g.off[e])
        indices = g.col[lo:hi].astype(np.int32)
        indptr = (g.off[s:e + 1] - lo).astype(np.int32)
        head = np.array([hi - lo, len(indices), len(indptr), s, e], np.int32)
        np.save(f"{d}{p}.edge.npy", np.concatenate([head, indices, indptr]).astype(np.int32))
    np.save(f"{d}vertexout.npy", np.ascontiguousarray(g.outdeg, np.int32))
    np.save(f"{d}vertexin.npy", np.diff(g.off).astype(np.int32))
    return d
