"""gx_pagerank_noalloc: PageRank for callers that cannot allocate device
memory (a plugin whose host application owns the GPU's allocator, a serving
path that may not allocate per request).  The caller hands in device
buffers; the library's scratch is a fixed array built into the library.

Checked through the C ABI against the engine's own PageRank entry point
(gx_run), on two calls in a row, within the PageRank tolerance of the other
parity tests.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import graphee_gb300 as gx

pytestmark = pytest.mark.gpu
PR_RTOL = 1e-5


def _p(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_matches_engine_on_two_calls():
    torch = pytest.importorskip("torch")
    g = gx.rmat_graph(16, 16, seed=33, P=4)
    with gx.Engine() as e:
        e.load(g)
        st = e.run(gx.APP_PAGERANK_REF, 20)
        ref = e.values().astype(np.float64)
    dev = torch.device("cuda", 0)
    off = torch.from_numpy(g.off).to(dev)
    col = torch.zeros(g.E + 4, dtype=torch.int32, device=dev)
    col[:g.E] = torch.from_numpy(g.col).to(dev)
    od = torch.from_numpy(g.outdeg).to(dev)
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
        assert steps.value == st["iterations"] == 20


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
