"""Parity of the CUDA path (through the C ABI) with the oracle and with the
reference's own outputs.  Bars: bit-exact for SSSP/CC values and for every
per-step `Update` count; PageRank bit-exact in exact-order mode, and within
1e-5 max relative error of the reference in the default (tree-reduced heavy
vertex) mode on R-MAT inputs."""
import numpy as np
import pytest

import graphee_gb300 as gx
import gx_oracle as O

pytestmark = pytest.mark.gpu

EXACT = {"exact_order": 1}
PR_RTOL = 1e-5


def engine_for(g, **cfg):
    e = gx.Engine(**cfg)
    e.load(g)
    return e


def golden_graph(c):
    return gx.Graph(int(c["V"]), c["off"], c["col"], c["outdeg"], int(c["P"]), c["bounds"])


def run_changed(e, steps):
    return np.array([e.iter_stats(i)["changed"] for i in range(steps)], np.int64)


@pytest.mark.parametrize("use_graph", [1, 0])
def test_pagerank_exact_order_bitexact_vs_reference(golden_cases, use_graph):
    for name, c in golden_cases.items():
        e = engine_for(golden_graph(c), use_graph=use_graph, **EXACT)
        st = e.run(gx.APP_PAGERANK_REF, 20)
        vals = e.values()
        assert np.array_equal(vals.view(np.uint32), c["pr"].view(np.uint32)), name
        assert st["iterations"] == len(c["pr_changed"]), name
        assert np.array_equal(run_changed(e, st["iterations"]), c["pr_changed"]), name
        e.close()


def test_pagerank_default_mode_vs_reference(golden_cases):
    for name, c in golden_cases.items():
        e = engine_for(golden_graph(c))
        e.run(gx.APP_PAGERANK_REF, 20)
        vals = e.values().astype(np.float64)
        ref = c["pr"].astype(np.float64)
        rel = np.abs(vals - ref) / np.abs(ref)
        # the hub fixture is where the reference's own sequential FP32 sum is ~2e-4 off FP64
        assert rel.max() < (1e-3 if name.startswith("hub") else PR_RTOL), (name, rel.max())
        e.close()


@pytest.mark.parametrize("push", [1, 0])
@pytest.mark.parametrize("source", [1, 0])
def test_sssp_unit_bitexact_vs_reference(golden_cases, push, source):
    for name, c in golden_cases.items():
        e = engine_for(golden_graph(c), push_sparse=push)
        st = e.run(gx.APP_SSSP, 200, source=source)
        assert np.array_equal(e.values(), c[f"sssp{source}"]), name
        assert np.array_equal(run_changed(e, st["iterations"]), c[f"sssp{source}_changed"]), name
        e.close()


@pytest.mark.parametrize("push", [1, 0])
def test_cc_bitexact_vs_reference(golden_cases, push):
    for name, c in golden_cases.items():
        e = engine_for(golden_graph(c), push_sparse=push)
        st = e.run(gx.APP_CC, 200)
        assert np.array_equal(e.values(), c["cc"]), name
        assert np.array_equal(run_changed(e, st["iterations"]), c["cc_changed"]), name
        e.close()


def test_pagerank_rmat16_vs_oracle():
    g = gx.rmat_graph(16, 16, seed=42, P=16)
    ref, ch, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 20)
    v64, _, _ = O.run(O.PAGERANK_REF64, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 20)
    e = engine_for(g)
    st = e.run(gx.APP_PAGERANK_REF, 20)
    vals = e.values().astype(np.float64)
    assert st["iterations"] == 20
    rel = np.abs(vals - ref) / np.abs(ref.astype(np.float64))
    assert rel.max() < PR_RTOL, rel.max()
    # L1 against FP64 is no worse than the reference's own
    assert np.abs(vals - v64).sum() <= 2 * np.abs(ref - v64).sum() + 1e-9
    ee = engine_for(g, **EXACT)
    ee.run(gx.APP_PAGERANK_REF, 20)
    assert np.array_equal(ee.values().view(np.uint32), ref.view(np.uint32))


def test_pagerank_std_vs_fp64():
    g = gx.rmat_graph(14, 16, seed=3, P=8)
    ref, _, _ = O.run(O.PAGERANK_STD, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 60)
    e = engine_for(g)
    st = e.run(gx.APP_PAGERANK_STD, 60)
    vals = e.values().astype(np.float64)
    # FP32 ranks become stationary before 60 steps, and then the reference's
    # stop rule (no vertex changed, GraphPS.h:383) ends the run.
    assert 20 < st["iterations"] <= 60
    assert e.iter_stats(st["iterations"] - 1)["changed"] == 0 or st["iterations"] == 60
    assert np.abs(vals - ref).sum() < 1e-5
    assert abs(vals.sum() - 1.0) < 1e-4
    # tolerance stop: L1 residual
    e.run(gx.APP_PAGERANK_STD, 500, tolerance=1e-6)
    its = e.run(gx.APP_PAGERANK_STD, 500, tolerance=1e-6)["iterations"]
    assert 5 < its < 500   # R-MAT PageRank residuals shrink ~4x per step
    assert e.iter_stats(its - 1)["residual_l1"] < 1e-6


# (push_sparse, push_edge_fraction): reference scheduling only, the default
# frontier-size rule, and push on every step.
PUSH_RULES = [(1, 0.5), (1, 0.0), (1, 1.0), (0, 0.5)]


@pytest.mark.parametrize("push,frac", PUSH_RULES)
def test_sssp_weighted_vs_oracle(push, frac):
    g = gx.rmat_graph(15, 16, seed=7, P=8, weight_seed=99)
    ref, ch, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000, weights=g.weights, source=0)
    e = engine_for(g, push_sparse=push, push_edge_fraction=frac)
    st = e.run(gx.APP_SSSP, 1000, source=0, weighted=True)
    assert np.array_equal(e.values(), ref)
    assert np.array_equal(run_changed(e, st["iterations"]), ch)
    if push:
        assert st["push_iterations"] > 0
    if push and frac == 1.0:
        assert st["push_iterations"] == st["iterations"]


@pytest.mark.parametrize("push,frac", PUSH_RULES)
def test_sssp_unit_and_cc_push_rules_vs_oracle(push, frac):
    g = gx.rmat_graph(14, 16, seed=21, P=8)
    ref, ch, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000, source=3)
    e = engine_for(g, push_sparse=push, push_edge_fraction=frac)
    st = e.run(gx.APP_SSSP, 1000, source=3)
    assert np.array_equal(e.values(), ref)
    assert np.array_equal(run_changed(e, st["iterations"]), ch)
    gs = gx.rmat_graph(14, 8, seed=22, P=8, symmetric=True)
    ref, ch, _ = O.run(O.CC, gs.V, gs.P, gs.bounds, gs.off, gs.col, gs.outdeg, 1000)
    e = engine_for(gs, push_sparse=push, push_edge_fraction=frac)
    st = e.run(gx.APP_CC, 1000)
    assert np.array_equal(e.values(), ref)
    assert np.array_equal(run_changed(e, st["iterations"]), ch)


def test_cc_symmetric_rmat_vs_oracle():
    g = gx.rmat_graph(15, 8, seed=12, P=8, symmetric=True)
    ref, ch, _ = O.run(O.CC, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000)
    e = engine_for(g)
    st = e.run(gx.APP_CC, 1000)
    assert np.array_equal(e.values(), ref)
    assert np.array_equal(run_changed(e, st["iterations"]), ch)


def test_indegree_app():
    g = gx.rmat_graph(12, 8, seed=2, P=4)
    ref, ch, _ = O.run(O.INDEGREE, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 10)
    e = engine_for(g)
    st = e.run(gx.APP_INDEGREE, 10)
    assert np.array_equal(e.values(), ref) and np.array_equal(e.values(), np.diff(g.off))
    assert st["iterations"] == len(ch) == 3


def test_streamed_shards_match_resident():
    """A shard-cache budget far below the graph forces the streaming ring.
    In exact-order mode both runs fold every list in edge order, so results
    are bit-identical; in the default mode the resident run sums medium and
    heavy vertices in a different (tree) order, so PageRank agrees to the
    PageRank tolerance and SSSP/CC stay bit-identical."""
    g = gx.rmat_graph(14, 16, seed=5, P=32, weight_seed=1)
    budget = g.E * 8 // 6
    for exact in (1, 0):
        res = engine_for(g, exact_order=exact)
        stm = engine_for(g, cache_budget_bytes=budget, stream_slots=2, exact_order=exact)
        for app, kw in [(gx.APP_PAGERANK_REF, {}), (gx.APP_SSSP, {"source": 0, "weighted": True}),
                        (gx.APP_CC, {})]:
            a = res.run(app, 30, **kw)
            b = stm.run(app, 30, **kw)
            va, vb = res.values(), stm.values()
            if exact or app != gx.APP_PAGERANK_REF:
                assert np.array_equal(va.view(np.uint32), vb.view(np.uint32)), (exact, app)
            else:
                assert np.abs(va.astype(np.float64) - vb).max() / va.max() < 1e-6
            assert a["iterations"] == b["iterations"]
            assert 0 < b["shards_resident"] < g.P and b["h2d_bytes"] > 0
        res.close()
        stm.close()


def test_load_shards_from_directory(tmp_path):
    g = gx.rmat_graph(11, 8, seed=1, P=4)
    d = gx.write_shards(g, tmp_path / "s")
    ps = gx.PagerankPS(**EXACT)
    ps.init(d, g.V, g.P, 20)
    ps.run()
    ref, _, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 20)
    assert np.array_equal(ps.vertex_msg.view(np.uint32), ref.view(np.uint32))
    s = gx.SsspPS()
    s.init(d, g.V, g.P, 100)
    s.run()
    ref, _, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 100, source=1)
    assert np.array_equal(s.vertex_msg, ref)


def test_set_init_and_errors():
    g = gx.rmat_graph(10, 8, seed=1, P=2)
    e = gx.Engine()
    with pytest.raises(gx.GxError) as ei:
        e.run(gx.APP_PAGERANK_REF, 5)
    assert ei.value.status == gx.GX_ERR_STATE
    e.load(g)
    with pytest.raises(gx.GxError) as ei:
        e.run(gx.APP_SSSP, 5, source=g.V)
    assert ei.value.status == gx.GX_ERR_INVALID
    with pytest.raises(gx.GxError) as ei:
        e.run(gx.APP_SSSP, 5, source=0, weighted=True)
    assert ei.value.status == gx.GX_ERR_STATE
    init = np.full(g.V, 1.0 / g.V, np.float32)
    init[:10] = 0.5
    e.set_init(init)
    e.run(gx.APP_PAGERANK_REF, 7, use_init=True)
    ref, _, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 7, init=init)
    assert np.abs(e.values() - ref).max() / ref.max() < 1e-5


def test_triangle_count_vs_oracle(golden_cases):
    for seed, scale in [(21, 12), (8, 15)]:
        g = gx.rmat_graph(scale, 16, seed=seed, P=4, symmetric=True)
        with engine_for(g) as e:
            t, st = e.triangle_count()
        assert t == O.triangles(g.V, g.off, g.col)
        assert st["edges_scanned"] > 0
    c = golden_cases["rmat12_sym_p8"]
    with engine_for(golden_graph(c)) as e:
        assert e.triangle_count()[0] == O.triangles(int(c["V"]), c["off"], c["col"])


def test_triangle_count_clique_uses_cta_path():
    """K_1200: every orientation list of the first vertices exceeds a warp's
    shared-memory slice, so the CTA path runs; C(1200, 3) triangles, plus a
    disjoint 4-cycle with a chord (2 triangles) and isolated vertices."""
    n = 1200
    iu = np.triu_indices(n, 1)
    src = np.concatenate([iu[0], [n, n + 1, n + 2, n + 3, n]])
    dst = np.concatenate([iu[1], [n + 1, n + 2, n + 3, n, n + 2]])
    V = n + 10
    off, col = gx.build_csc(V, src.astype(np.int32), dst.astype(np.int32),
                            gx.BUILD_DROP_SELF | gx.BUILD_DEDUP | gx.BUILD_SYMMETRIZE)
    g = gx.Graph(V, off, col, None, 3)
    with engine_for(g) as e:
        t, _ = e.triangle_count()
    assert t == n * (n - 1) * (n - 2) // 6 + 2


def test_triangle_count_empty_graph():
    g = gx.Graph(16, np.zeros(17, np.int64), np.zeros(0, np.int32), None, 2)
    with engine_for(g) as e:
        assert e.triangle_count()[0] == 0


@pytest.mark.parametrize("k", [64, 8, 5, 1])
def test_ppr_vs_fp64(k):
    g = gx.rmat_graph(13, 16, seed=17, P=4)
    rng = np.random.default_rng(k)
    src = rng.integers(0, g.V, size=k).astype(np.int32)
    src[0] = int(np.argmax(np.diff(g.off)))       # a hub source (chunked rows)
    ref = O.ppr(g.V, g.off, g.col, g.outdeg, src, 15, 0.15)
    with engine_for(g) as e:
        R, st = e.ppr(src, 15)
        R2, _ = e.ppr(src, 15)
    assert np.array_equal(R, R2)                   # deterministic
    assert np.abs(R - ref).max() < 1e-6
    assert np.all(np.abs(R - ref).sum(axis=0) < 1e-5 * np.maximum(1.0, ref.sum(axis=0)))
    assert st["iterations"] == 15
    assert st["kernel_launches"] == 2          # one init kernel, one persistent launch for all 15 steps


def _instance(g, vb, i):
    b, e = int(vb[i]), int(vb[i + 1])
    off = g.off[b:e + 1] - g.off[b]
    col = g.col[g.off[b]:g.off[e]] - b
    return e - b, off, col, g.outdeg[b:e]


def test_batched_pagerank_cc_vs_oracle(tmp_path):
    g, vb = gx.batch_graph(40, scales=(5, 11), edge_factors=(2, 16), seed=3)
    with engine_for(g) as e:
        pr, cc, ps, cs, st = e.batch_run(vb, pr_iters=30, cc_max_iter=1000)
        best, ms = e.batch_autotune(vb, pr_iters=30, cc_max_iter=1000, table_path=tmp_path / "tune.jsonl")
        pr2, cc2, _, _, _ = e.batch_run(vb, pr_iters=30, cc_max_iter=1000, tuning=best)
    assert st["kernel_launches"] == 1 and ms > 0
    assert (tmp_path / "tune.jsonl").read_text().count("candidates") == 1
    for i in range(len(vb) - 1):
        n, off, col, od = _instance(g, vb, i)
        b = np.array([0, n], np.int32)
        ref, ch, _ = O.run(O.PAGERANK_REF, n, 1, b, off, col, od, 30)
        sl = slice(vb[i], vb[i + 1])
        assert np.abs(pr[sl] - ref).max() / ref.max() < 1e-5, i
        assert ps[i] == len(ch)
        lab, chc, _ = O.run(O.CC, n, 1, b, off, col, od, 1000)
        assert np.array_equal(cc[sl], lab), i
        assert cs[i] == len(chc)
    assert np.array_equal(cc, cc2) and np.abs(pr - pr2).max() < 1e-6


def test_batch_rejects_cross_instance_edges():
    g, vb = gx.batch_graph(4, scales=(5, 6), edge_factors=(4, 4), seed=1)
    bad = vb.copy()
    bad[2] = bad[2] + 3           # instance boundaries no longer match the edges
    with engine_for(g) as e:
        with pytest.raises(gx.GxError) as ei:
            e.batch_run(bad)
    assert ei.value.status == gx.GX_ERR_INVALID


def test_cpp_app_drivers_vs_oracle(tmp_path):
    """The C++ GraphPS<T> mirror (include/gx_graphps.hpp) behind the
    command-line drivers, on shards written in the reference layout."""
    import subprocess
    g = gx.rmat_graph(12, 16, seed=4, P=6)
    d = gx.write_shards(g, tmp_path / "s")
    app = str(gx.LIB_PATH.parent / "gx_app")
    out = tmp_path / "pr.bin"
    subprocess.run([app, "pagerank", d, str(g.V), str(g.P), "20", str(out)], check=True)
    ref, _, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 20)
    vals = np.fromfile(out, np.float32)
    assert np.abs(vals - ref).max() / ref.max() < 1e-5
    subprocess.run([app, "sssp", d, str(g.V), str(g.P), "100", str(out), "0"], check=True)
    ref, _, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 100, source=0)
    assert np.array_equal(np.fromfile(out, np.int32), ref)
    s = gx.rmat_graph(11, 8, seed=5, P=3, symmetric=True)
    d2 = gx.write_shards(s, tmp_path / "t")
    r = subprocess.run([app, "tc", d2, str(s.V), str(s.P), "0"], check=True, capture_output=True, text=True)
    assert int(r.stdout.strip()) == O.triangles(s.V, s.off, s.col)


@pytest.mark.parametrize("budget,relabel", [(-1, 0), (1 << 20, 0), (-1, 1)])
def test_load_rejects_bad_csc(budget, relabel):
    g = gx.rmat_graph(10, 8, seed=3, P=4)
    col = g.col.copy()
    col[17] = g.V + 5
    bad = gx.Graph(g.V, g.off, col, g.outdeg, g.P, g.bounds)
    with gx.Engine(cache_budget_bytes=budget, relabel=relabel) as e:
        with pytest.raises(gx.GxError) as ei:
            e.load(bad)
        assert ei.value.status == gx.GX_ERR_INVALID and "source id" in str(ei.value)
        off = g.off.copy()
        off[100], off[101] = off[101], off[100] - 1
        with pytest.raises(gx.GxError) as ei:
            e.load(gx.Graph(g.V, off, g.col, g.outdeg, g.P, g.bounds))
        assert ei.value.status == gx.GX_ERR_INVALID
        e.load(g)                      # the engine is still usable
        assert e.run(gx.APP_CC, 100)["iterations"] > 0


def test_selective_steps_skip_shards_and_keep_values():
    """On a path the SSSP frontier is one vertex per step, far below BF_THRE:
    with push steps off, every step after the first few is selective, and
    once the out-edge CSR that marks shards is built (at the first selective
    step, seen by the host after a replay of 8 steps) a step sweeps exactly
    the one shard that holds the frontier's out-neighbour.  Values and
    per-step counts stay the reference's."""
    V = 4096
    src = np.arange(V - 1, dtype=np.int32)
    off, col = gx.build_csc(V, src, src + 1)
    g = gx.Graph(V, off, col, None, 16)
    ref, ch, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 5000, source=0)
    e = engine_for(g, push_sparse=0)
    st = e.run(gx.APP_SSSP, 5000, source=0)
    assert np.array_equal(e.values(), ref)
    assert np.array_equal(run_changed(e, st["iterations"]), ch)
    stats = [e.iter_stats(i) for i in range(st["iterations"])]
    e.close()
    sel = [(t, m) for t, m in enumerate(stats) if m["mode"] == 1]
    assert len(sel) > V // 2
    # one shard per step (none after the last vertex, which has no out-edge)
    for t, m in sel[16:]:
        assert m["shards_active"] == len(_frontier_shards(g, ref, t)) <= 1, t
    assert sum(m["shards_active"] == 1 for _, m in sel) > V // 2


def _frontier_shards(g, dist, t):
    """Shards holding the out-neighbours of the vertices unit-weight SSSP
    changes at step t - 1 (those at distance t)."""
    dst = np.repeat(np.arange(g.V), np.diff(g.off))
    src_at_t = dist[g.col] == t
    return set((np.searchsorted(g.bounds, dst[src_at_t], side="right") - 1).tolist())


@pytest.mark.parametrize("budget", [-1, "stream"])
def test_selective_steps_sweep_exactly_the_marked_shards(budget):
    """A broom (8 paths of 2,000 vertices hanging off vertex 0) in 256
    shards: 8 vertices change per step, so every step after the first few is
    selective, and each one sweeps exactly the shards that hold the last
    step's changed vertices' out-neighbours (the partition activation of
    GraphMP/system/GraphPS.h:349-368, exact per shard).  Resident graphs mark
    them on the device from the out-edge CSR; streamed graphs list the changed
    vertices for the host.  Values and per-step counts stay the reference's."""
    k, L = 8, 2000
    src, dst = [], []
    for j in range(k):
        head = 1 + j * L
        src += [0] + list(range(head, head + L - 1))
        dst += [head] + list(range(head + 1, head + L))
    V = 1 + k * L
    off, col = gx.build_csc(V, np.array(src, np.int32), np.array(dst, np.int32))
    g = gx.Graph(V, off, col, None, 256)
    ref, ch, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 5000, source=0)
    cfg = {"push_sparse": 0}
    if budget == "stream":
        cfg.update(cache_budget_bytes=g.E * 4 // 3, stream_slots=2)
    with engine_for(g, **cfg) as e:
        st = e.run(gx.APP_SSSP, 5000, source=0)
        assert np.array_equal(e.values(), ref)
        assert np.array_equal(run_changed(e, st["iterations"]), ch)
        stats = [e.iter_stats(i) for i in range(st["iterations"])]
    checked = 0
    for t, m in enumerate(stats):
        if m["mode"] != 1 or m["shards_active"] == g.P or t < 2:
            continue
        assert m["shards_active"] == len(_frontier_shards(g, ref, t)), t
        checked += 1
    assert checked > L // 2


@pytest.mark.parametrize("budget,relabel", [(-1, 0), (0, 0), (-1, 1)])
def test_graph_without_edges(budget, relabel):
    """No edges at all (every shard empty): the apps still follow the
    reference's loop and stop rule, resident, relabelled or with a zero
    budget."""
    V, P = 100, 4
    g = gx.Graph(V, np.zeros(V + 1, np.int64), np.zeros(0, np.int32), None, P)
    for app, kw, oapp in [(gx.APP_PAGERANK_REF, {}, O.PAGERANK_REF), (gx.APP_SSSP, {"source": 0}, O.SSSP),
                          (gx.APP_CC, {}, O.CC)]:
        ref, ch, _ = O.run(oapp, V, P, g.bounds, g.off, g.col, g.outdeg, 50, **kw)
        with gx.Engine(cache_budget_bytes=budget, relabel=relabel) as e:
            e.load(g)
            st = e.run(app, 50, **kw)
            assert np.array_equal(e.values().view(np.uint32), ref.view(np.uint32)), app
            assert np.array_equal(run_changed(e, st["iterations"]), ch), app


def test_cached_superstep_graphs_follow_the_loaded_graph():
    """gx_run replays an executable graph captured by an earlier run with the
    same kernels, launch shapes and argument bytes.  Runs of different apps
    and lengths, and a second graph of the same size loaded into the same
    engine, all match the oracle."""
    g1 = gx.rmat_graph(14, 16, seed=61, P=8, weight_seed=3)
    g2 = gx.rmat_graph(14, 16, seed=62, P=8, weight_seed=4)
    with gx.Engine(exact_order=1) as e:
        for g in (g1, g2, g1):
            e.load(g)
            for iters in (20, 5, 20):
                e.run(gx.APP_PAGERANK_REF, iters)
                ref, _, _ = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, iters)
                assert np.array_equal(e.values().view(np.uint32), ref.view(np.uint32)), iters
            e.run(gx.APP_SSSP, 1000, source=0, weighted=True)
            ref, _, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000, weights=g.weights, source=0)
            assert np.array_equal(e.values(), ref)
