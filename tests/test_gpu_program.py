"""Vertex programs plugged in from outside the library (include/gx_program.cuh,
compiled in graphee_gb300/apps/gx_program_example.cu against the headers and
libgx.so), the plug-in point that GraphPS<T>'s _comp and init_vertex() are in
the reference (GraphMP/system/GraphPS.h:25-34,60): min-label CC, unit SSSP
from vertex 0 and PageRank re-expressed as plug-ins match the oracle (CC and
SSSP bit-exact with per-step counts, PageRank within 1e-5), and a program the
engine does not ship (widest path) matches a numpy restatement."""
import ctypes as C

import numpy as np
import pytest

import graphee_gb300 as gx
import gx_oracle as O

pytestmark = pytest.mark.gpu

MIN_LABEL, HOPS, PAGERANK, WIDEST = range(4)


def example():
    L = C.CDLL(str(gx.LIB_PATH.parent / "libgx_program_example.so"))
    L.gx_example_program.restype = C.c_int
    L.gx_example_program.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    return L


def run(e, which, max_iter, dtype, V):
    out = np.empty(V, dtype)
    changed = np.zeros(max_iter, np.int64)
    steps = C.c_int32(0)
    rc = example().gx_example_program(e._h, which, max_iter, out.ctypes.data_as(C.c_void_p),
                                      changed.ctypes.data_as(C.c_void_p), C.byref(steps))
    assert rc == gx.GX_OK, gx.lib().gx_last_error()
    return out, changed[:steps.value]


def test_plugged_cc_and_sssp_match_oracle():
    g = gx.rmat_graph(15, 8, seed=31, P=8, symmetric=True)
    ref, ch, _ = O.run(O.CC, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000)
    with gx.Engine() as e:
        e.load(g)
        vals, got = run(e, MIN_LABEL, 1000, np.int32, g.V)
    assert np.array_equal(vals, ref) and np.array_equal(got, ch)
    d = gx.rmat_graph(15, 16, seed=32, P=8)
    ref, ch, _ = O.run(O.SSSP, d.V, d.P, d.bounds, d.off, d.col, d.outdeg, 1000, source=0)
    with gx.Engine() as e:
        e.load(d)
        vals, got = run(e, HOPS, 1000, np.int32, d.V)
    assert np.array_equal(vals, ref) and np.array_equal(got, ch)


def test_plugged_pagerank_within_tolerance():
    g = gx.rmat_graph(16, 16, seed=33, P=8)
    ref, ch, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 20)
    with gx.Engine() as e:
        e.load(g)
        vals, got = run(e, PAGERANK, 20, np.float32, g.V)
    assert len(got) == len(ch) == 20
    assert np.max(np.abs(vals.astype(np.float64) - ref) / ref) < 1e-5


def test_plugged_widest_path_matches_numpy():
    g = gx.rmat_graph(13, 16, seed=34, P=4, weight_seed=9)
    dst = np.repeat(np.arange(g.V), np.diff(g.off))
    d = np.zeros(g.V, np.uint64)
    d[0] = 0xFFFFFFFF
    changed = []
    prev = np.zeros(g.V, np.uint64)            # VertexValue before the first step
    for step in range(1000):
        cand = np.zeros(g.V, np.uint64)
        np.maximum.at(cand, dst, np.minimum(d[g.col], g.weights.astype(np.uint64)))
        nd = np.maximum(d, cand)
        changed.append(int(np.sum(nd != (prev if step == 0 else d))))
        d = nd
        if changed[-1] == 0 and step > 1:
            break
    with gx.Engine() as e:
        e.load(g)
        vals, got = run(e, WIDEST, 1000, np.uint32, g.V)
    assert np.array_equal(vals.astype(np.uint64), d)
    assert list(got) == changed


def test_device_graph_needs_resident_shards():
    g = gx.rmat_graph(12, 16, seed=35, P=8)
    with gx.Engine(cache_budget_bytes=g.E) as e:       # a quarter of the edge bytes: shards stream
        e.load(g)
        out = np.empty(g.V, np.int32)
        rc = example().gx_example_program(e._h, MIN_LABEL, 10, out.ctypes.data_as(C.c_void_p), None, None)
        assert rc == gx.GX_ERR_STATE
