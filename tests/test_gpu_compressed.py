"""The compressed shard cache: with a budget the plain shards exceed, every
shard is kept as per-chunk offsets (and byte weights) and decoded in the
pull kernel, which otherwise reads and folds exactly as on plain shards.
Values and per-step counts equal the resident run's bit for bit in both
modes, and fewer bytes are streamed than through the plain ring."""
import numpy as np
import pytest

import graphee_gb300 as gx
import gx_oracle as O

pytestmark = pytest.mark.gpu

APPS = [(gx.APP_PAGERANK_REF, {}, False), (gx.APP_SSSP, {"source": 0, "weighted": True}, False),
        (gx.APP_SSSP, {"source": 3}, False), (gx.APP_CC, {}, True)]


def engine(g, **cfg):
    e = gx.Engine(**cfg)
    e.load(g)
    return e


def changed(e, n):
    return [e.iter_stats(i)["changed"] for i in range(n)]


def same(app, exact, va, vb):
    return np.array_equal(va.view(np.uint32), vb.view(np.uint32))


@pytest.mark.parametrize("exact", [0, 1])
@pytest.mark.parametrize("app,kw,sym", APPS)
def test_compressed_matches_resident(app, kw, sym, exact):
    g = gx.rmat_graph(15, 16, seed=9, P=32, symmetric=sym, weight_seed=4)
    res = engine(g, exact_order=exact)
    a = res.run(app, 40, **kw)
    va = res.values().copy()
    budget = g.E * 2                      # below the plain shards, about half the compressed ones
    comp = engine(g, cache_budget_bytes=budget, stream_slots=3, exact_order=exact)
    b = comp.run(app, 40, **kw)
    assert same(app, exact, va, comp.values())
    assert a["iterations"] == b["iterations"]
    assert changed(res, a["iterations"]) == changed(comp, b["iterations"])
    assert 0 < b["shards_resident"] < g.P and b["shards_streamed"] > 0
    plain = engine(g, cache_budget_bytes=budget, stream_slots=3, compress_cache=0, exact_order=exact)
    c = plain.run(app, 40, **kw)
    assert same(app, exact, va, plain.values())
    # Per streamed shard the compressed blob is smaller, and more shards stay resident.
    assert b["h2d_bytes"] < c["h2d_bytes"]
    for e in (res, comp, plain):
        e.close()


def test_compressed_weighted_sssp_and_wide_weights():
    g = gx.rmat_graph(14, 16, seed=2, P=16, weight_seed=8)
    raw = g.E * 8
    ref, ch, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000, weights=g.weights, source=0)
    # Most shards resident (plain), the rest streamed compressed with byte weights.
    with gx.Engine(cache_budget_bytes=int(raw * 0.8)) as e:
        e.load(g)
        st = e.run(gx.APP_SSSP, 1000, source=0, weighted=True)
        assert np.array_equal(e.values(), ref) and changed(e, st["iterations"]) == list(ch)
        assert 0 < st["shards_resident"] < g.P and st["shards_streamed"] > 0
    # Weights above 255 do not fit a byte: the plain ring is used.
    w = g.weights.astype(np.uint32) * 300
    ref2, _, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000, weights=w, source=0)
    g2 = gx.Graph(g.V, g.off, g.col, g.outdeg, g.P, g.bounds, w)
    with gx.Engine(cache_budget_bytes=g.E * 2) as e:
        e.load(g2)
        st = e.run(gx.APP_SSSP, 1000, source=0, weighted=True)
        assert np.array_equal(e.values(), ref2)


def test_compressed_zero_width_chunks():
    # Vertex 0 feeds 5000 vertices of in-degree 1: chunks of 32 equal ids (width 0),
    # next to random lists (wide chunks).
    V = 8192
    rng = np.random.default_rng(3)
    src = np.concatenate([np.zeros(5000, np.int32), rng.integers(0, V, 60000, dtype=np.int32)])
    dst = np.concatenate([np.arange(1, 5001, dtype=np.int32), rng.integers(5001, V, 60000, dtype=np.int32)])
    off, col = gx.build_csc(V, src, dst)
    g = gx.Graph(V, off, col, None, 8)
    res = engine(g)
    res.run(gx.APP_PAGERANK_REF, 15)
    comp = engine(g, cache_budget_bytes=g.E)
    st = comp.run(gx.APP_PAGERANK_REF, 15)
    assert st["shards_streamed"] > 0
    assert same(gx.APP_PAGERANK_REF, 0, res.values(), comp.values())
    res.close()
    comp.close()
