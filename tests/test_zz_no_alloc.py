"""gx_pagerank_noalloc: PageRank for callers that cannot allocate device
memory (a plugin whose host application owns the GPU's allocator, a serving
path that may not allocate per request).  The caller hands in device
buffers; the library's scratch is a fixed array built into the library.

Checked through the C ABI against the oracle's restatement of the
reference's PageRank (GraphMP/app/pagerank.cpp:42-60), on two calls in a
row, within the PageRank tolerance of the other parity tests, on an R-MAT
graph with vertices of more than 4,096 in-edges (the entry point sweeps
every list with the tile's warp, hubs included).  A CSC that fails the
entry point's device-side checks is refused without running a superstep.
This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import graphee_gb300 as gx
import gx_oracle as O

pytestmark = pytest.mark.gpu
PR_RTOL = 1e-5


def _p(t):
    return C.c_void_p(t.data_ptr())


def _device_csc(torch, g):
    dev = torch.device("cuda", 0)
    off = torch.from_numpy(g.off).to(dev)
    col = torch.zeros(g.E + 4, dtype=torch.int32, device=dev)
    col[:g.E] = torch.from_numpy(g.col).to(dev)
    od = torch.from_numpy(g.outdeg).to(dev)
    return dev, off, col, od


def test_noalloc_matches_oracle_on_two_calls():
    torch = pytest.importorskip("torch")
    g = gx.rmat_graph(17, 16, seed=33, P=4)
    assert (np.diff(g.off) > 4096).sum() > 0          # hubs beyond the engine's heavy threshold
    ref, ch, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 20)
    r64, _, _ = O.run(O.PAGERANK_REF64, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 20)
    ref = ref.astype(np.float64)
    dev, off, col, od = _device_csc(torch, g)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    for call in range(2):
        rank = torch.full((g.V,), -1.0, dtype=torch.float32, device=dev)
        steps = C.c_int32(0)
        rc = gx.lib().gx_pagerank_noalloc(_p(off), _p(col), g.E, g.E + 4, _p(od), g.V, 20, 0.85, _p(rank), stream,
                                          C.byref(steps))
        assert rc == gx.GX_OK, gx.lib().gx_last_error()
        vals = rank.cpu().numpy().astype(np.float64)
        rel = np.abs(vals - ref) / ref
        assert rel.max() < PR_RTOL, (call, rel.max())
        assert np.abs(vals - r64).sum() <= 2 * np.abs(ref - r64).sum()
        assert steps.value == len(ch) == 20


def test_noalloc_rejects_a_bad_csc_without_running():
    torch = pytest.importorskip("torch")
    g = gx.rmat_graph(12, 8, seed=5, P=1)
    dev, off, col, od = _device_csc(torch, g)
    col[g.E // 2] = g.V                              # one source id out of range
    rank = torch.full((g.V,), -1.0, dtype=torch.float32, device=dev)
    steps = C.c_int32(-1)
    L = gx.lib()
    rc = L.gx_pagerank_noalloc(_p(off), _p(col), g.E, g.E + 4, _p(od), g.V, 10, 0.85, _p(rank), None,
                               C.byref(steps))
    assert rc == gx.GX_ERR_INVALID and b"device-side checks" in L.gx_last_error()
    assert steps.value == 0
    r = rank.cpu().numpy()
    assert np.all(r == np.float32(1.0 / g.V))         # the start value: no superstep touched it
    col[g.E // 2] = int(g.col[g.E // 2])
    off_bad = off.clone()
    off_bad[-1] = g.E - 1                             # off[V] != num_edges
    rc = L.gx_pagerank_noalloc(_p(off_bad), _p(col), g.E, g.E + 4, _p(od), g.V, 10, 0.85, _p(rank), None,
                               C.byref(steps))
    assert rc == gx.GX_ERR_INVALID
    rc = L.gx_pagerank_noalloc(_p(off), _p(col), g.E, g.E + 4, _p(od), g.V, 10, 0.85, _p(rank), None,
                               C.byref(steps))
    assert rc == gx.GX_OK and steps.value == 10
    ref, _, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 10)
    assert np.abs(rank.cpu().numpy() - ref).max() / ref.max() < PR_RTOL


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.int64, device=dev)
    ptr = _p(buf)
    L = gx.lib()
    rc = L.gx_pagerank_noalloc(ptr, ptr, 0, 4, ptr, (1 << 20) + 1, 10, 0.85, ptr, None, None)
    assert rc == gx.GX_ERR_INVALID and b"scratch" in L.gx_last_error()
    rc = L.gx_pagerank_noalloc(ptr, ptr, 0, 4, ptr, 8, 1025, 0.85, ptr, None, None)
    assert rc == gx.GX_ERR_INVALID
    rc = L.gx_pagerank_noalloc(ptr, ptr, 10, 12, ptr, 8, 10, 0.85, ptr, None, None)
    assert rc == gx.GX_ERR_INVALID and b"num_edges + 4" in L.gx_last_error()
