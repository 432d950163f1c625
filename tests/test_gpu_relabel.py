"""The engine's relabelled layout (config.relabel): within every shard the
vertices are renumbered by descending in-degree, each keeping its in-list in
the caller's order with renamed sources.  Everything at the boundary stays in
the caller's numbering, so every result must equal the plain engine's and the
oracle's: PageRank bit-exact in exact-order mode with the per-step `Update`
counts, the default mode within 1e-5 of the reference's ranks and of the
plain engine's, SSSP (weighted
and unit) and CC values and counts bit-exact, start values, checkpoints and
resumed runs, PPR rows, triangle counts and the warm-start predictions."""
import ctypes as C

import numpy as np
import pytest

import graphee_gb300 as gx
import gx_oracle as O
import gx_mlp_oracle as MO

pytestmark = pytest.mark.gpu

RL = {"relabel": 1}


def counts(e, steps):
    return np.array([e.iter_stats(i)["changed"] for i in range(steps)], np.int64)


@pytest.fixture(scope="module")
def rmat16():
    return gx.rmat_graph(16, 16, seed=41, P=32, weight_seed=7)


def golden_graph(c):
    return gx.Graph(int(c["V"]), c["off"], c["col"], c["outdeg"], int(c["P"]), c["bounds"])


def test_reference_golden_vectors(golden_cases):
    """The reference's own outputs (its compiled apps on the fixtures: R-MAT,
    a path, a 3000-in-edge hub, components with self-loops and isolated
    vertices, empty shards), reproduced by a relabelled engine: PageRank in
    exact-order mode, SSSP from vertices 1 and 0 (push on and off) and CC,
    values and per-step counts bit for bit."""
    for name, c in golden_cases.items():
        g = golden_graph(c)
        with gx.Engine(exact_order=1, **RL) as e:
            e.load(g)
            st = e.run(gx.APP_PAGERANK_REF, 20)
            assert np.array_equal(e.values().view(np.uint32), c["pr"].view(np.uint32)), name
            assert np.array_equal(counts(e, st["iterations"]), c["pr_changed"]), name
        for push in (1, 0):
            with gx.Engine(push_sparse=push, **RL) as e:
                e.load(g)
                for source in (1, 0):
                    st = e.run(gx.APP_SSSP, 200, source=source)
                    assert np.array_equal(e.values(), c[f"sssp{source}"]), (name, push, source)
                    assert np.array_equal(counts(e, st["iterations"]), c[f"sssp{source}_changed"]), (name, push)
                st = e.run(gx.APP_CC, 200)
                assert np.array_equal(e.values(), c["cc"]), (name, push)
                assert np.array_equal(counts(e, st["iterations"]), c["cc_changed"]), (name, push)


@pytest.mark.parametrize("P", [1, 1024])
def test_one_shard_and_tiny_shards(P):
    """One shard (the whole graph renumbered as one) and shards of four
    vertices: PageRank exact-order, weighted SSSP and CC bit-exact."""
    g = gx.rmat_graph(12, 16, seed=5, P=P, weight_seed=3)
    ref, ch, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 20)
    dist, dch, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000, weights=g.weights, source=0)
    with gx.Engine(exact_order=1, **RL) as e:
        e.load(g)
        st = e.run(gx.APP_PAGERANK_REF, 20)
        assert np.array_equal(e.values().view(np.uint32), ref.view(np.uint32))
        assert np.array_equal(counts(e, st["iterations"]), ch)
        e.set_weights(g.weights)
        st = e.run(gx.APP_SSSP, 1000, source=0, weighted=True)
        assert np.array_equal(e.values(), dist)
        assert np.array_equal(counts(e, st["iterations"]), dch)
    gs = gx.rmat_graph(12, 8, seed=6, P=P, symmetric=True)
    lab, lch, _ = O.run(O.CC, gs.V, gs.P, gs.bounds, gs.off, gs.col, gs.outdeg, 1000)
    with gx.Engine(**RL) as e:
        e.load(gs)
        st = e.run(gx.APP_CC, 1000)
        assert np.array_equal(e.values(), lab)
        assert np.array_equal(counts(e, st["iterations"]), lch)


def test_pagerank_exact_order_bitexact(rmat16):
    g = rmat16
    ref, ch, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 20)
    with gx.Engine(exact_order=1, **RL) as e:
        e.load(g)
        st = e.run(gx.APP_PAGERANK_REF, 20)
        assert np.array_equal(e.values().view(np.uint32), ref.view(np.uint32))
        assert np.array_equal(counts(e, st["iterations"]), ch)


def test_pagerank_default_mode_matches_plain_engine(rmat16):
    g = rmat16
    ref, _, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 20)
    with gx.Engine(**RL) as e:
        e.load(g)
        e.run(gx.APP_PAGERANK_REF, 20)
        got = e.values().copy()
    with gx.Engine() as e:
        e.load(g)
        e.run(gx.APP_PAGERANK_REF, 20)
        plain = e.values().copy()
    assert np.abs(got.astype(np.float64) - ref).max() / ref.max() < 1e-5
    # The default mode tree-reduces a list in a shape that depends on where
    # the list falls in its sweep, so the two layouts round differently (an
    # ulp here and there), within the same bar.
    assert (np.abs(got.astype(np.float64) - plain) / plain).max() < 1e-5


def test_pagerank_std_matches_plain_engine(rmat16):
    g = rmat16
    out = []
    for cfg in ({}, RL):
        with gx.Engine(**cfg) as e:
            e.load(g)
            st = e.run(gx.APP_PAGERANK_STD, 200, tolerance=1e-7)
            out.append((e.values().copy(), st["iterations"]))
    assert out[0][1] == out[1][1]
    assert np.abs(out[0][0].astype(np.float64) - out[1][0]).sum() < 1e-6


@pytest.mark.parametrize("push", [1, 0])
def test_sssp_weighted_and_unit_bitexact(rmat16, push):
    g = rmat16
    for weighted, source in [(True, 0), (False, 5)]:
        ref, ch, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000,
                           weights=g.weights if weighted else None, source=source)
        with gx.Engine(push_sparse=push, **RL) as e:
            e.load(g)
            st = e.run(gx.APP_SSSP, 1000, source=source, weighted=weighted)
            assert np.array_equal(e.values(), ref)
            assert np.array_equal(counts(e, st["iterations"]), ch)


@pytest.mark.parametrize("async_mode", [False, True])
def test_cc_bitexact(async_mode):
    g = gx.rmat_graph(15, 8, seed=12, P=8, symmetric=True)
    ref, ch, _ = O.run(O.CC, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000)
    with gx.Engine(**RL) as e:
        e.load(g)
        st = e.run(gx.APP_CC, 1000, async_mode=async_mode)
        assert np.array_equal(e.values(), ref)
        if not async_mode:
            assert np.array_equal(counts(e, st["iterations"]), ch)


def test_start_values_checkpoint_and_resume(tmp_path, rmat16):
    g = rmat16
    init = np.full(g.V, 1.0 / g.V, np.float32)
    init[:10] = 0.5
    ref, _, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 7, init=init)
    with gx.Engine(exact_order=1, **RL) as e:
        e.load(g)
        e.set_init(init)
        e.run(gx.APP_PAGERANK_REF, 7, use_init=True)
        assert np.array_equal(e.values().view(np.uint32), ref.view(np.uint32))
        full = e.run(gx.APP_SSSP, 200, source=0, weighted=True, checkpoint_every=2,
                     checkpoint_prefix=str(tmp_path / "ck_"))
        final = e.values().copy()
        steps = full["iterations"]
        k = 2
        assert steps > k
        dist, _, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, k, weights=g.weights, source=0)
        ck = gx.read_values(tmp_path / f"ck_{k}.npy", g.V)
        assert np.array_equal(ck.view(np.uint32), dist.view(np.uint32))   # checkpoints in the caller's numbering
        e.set_init(ck)
        res = e.run(gx.APP_SSSP, 200, source=0, weighted=True, use_init=True, first_step=k)
        assert res["iterations"] == steps
        assert np.array_equal(e.values(), final)


def test_ppr_rows_and_triangles():
    g = gx.rmat_graph(13, 16, seed=17, P=4)
    rng = np.random.default_rng(8)
    src = rng.integers(0, g.V, size=8).astype(np.int32)
    src[0] = int(np.argmax(np.diff(g.off)))
    ref = O.ppr(g.V, g.off, g.col, g.outdeg, src, 15, 0.15)
    with gx.Engine(**RL) as e:
        e.load(g)
        R, _ = e.ppr(src, 15)
    assert np.abs(R - ref).max() < 1e-6
    gs = gx.rmat_graph(14, 16, seed=8, P=4, symmetric=True)
    with gx.Engine(**RL) as e:
        e.load(gs)
        assert e.triangle_count()[0] == O.triangles(gs.V, gs.off, gs.col)


def test_warm_start_prediction_in_caller_numbering():
    g = gx.rmat_graph(14, 16, seed=11, P=4)
    m = gx.MLP(seed=6)
    p, _ = m.params()
    rng = np.random.default_rng(2)
    p = (p + rng.normal(0, 0.05, size=p.shape)).astype(np.float32)
    F = MO.features(g.V, g.off, g.col, g.outdeg)
    norm = np.concatenate([F.mean(0), 1.0 / (F.std(0) + 1e-6)]).astype(np.float32)
    m.set_params(p, norm)
    with gx.Engine(**RL) as e:
        e.load(g)
        pred, _ = m.predict(e)
        ws = e.pagerank_warm(m, 300, tolerance=1e-7)
        warm = e.values().copy()
    ref = MO.predict(p, norm, F)
    ref = ref / ref.sum()
    assert np.abs(pred.astype(np.float64) - ref).sum() < 5e-3
    pr, _, _ = O.run(O.PAGERANK_STD, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 300)
    assert ws["iterations"] > 0 and np.abs(warm.astype(np.float64) - pr).sum() < 1e-5


def test_batch_and_device_graph_refuse_a_relabelled_engine():
    g, vb = gx.batch_graph(4, scales=(5, 6), edge_factors=(4, 4), seed=1)
    with gx.Engine(**RL) as e:
        e.load(g)
        with pytest.raises(gx.GxError) as ei:
            e.batch_run(vb)
        assert ei.value.status == gx.GX_ERR_STATE
        # A plug-in program sees the device graph, which is not in the
        # caller's numbering: the accessor refuses.
        L = C.CDLL(str(gx.LIB_PATH.parent / "libgx_program_example.so"))
        L.gx_example_program.restype = C.c_int
        L.gx_example_program.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
        assert L.gx_example_program(e._h, 0, 10, None, None, None) == gx.GX_ERR_STATE


def test_budgeted_load_keeps_the_caller_numbering():
    """With a shard-cache budget the option has no effect (the host keeps the
    streaming source in the caller's layout)."""
    g = gx.rmat_graph(14, 16, seed=31, P=16)
    ref, ch, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 10)
    with gx.Engine(cache_budget_bytes=1 << 20, exact_order=1, **RL) as e:
        e.load(g)
        st = e.run(gx.APP_PAGERANK_REF, 10)
        assert np.array_equal(e.values().view(np.uint32), ref.view(np.uint32))
        assert np.array_equal(counts(e, st["iterations"]), ch)
