"""Checkpoint/resume of vertex state and the Gauss-Seidel (async) mode.

A run resumed from a checkpoint with `first_step` continues the interrupted
run exactly: same values (bit for bit) and the same per-step counts for the
remaining steps.  Async mode (GraphH's USE_ASYNC) changes the step structure
but not the fixed point: SSSP distances and CC labels equal the oracle's."""
import numpy as np
import pytest

import graphee_gb300 as gx
import gx_oracle as O

pytestmark = pytest.mark.gpu


def changed(e, lo, hi):
    return [e.iter_stats(i)["changed"] for i in range(lo, hi)]


@pytest.mark.parametrize("app,weighted,budget", [(gx.APP_PAGERANK_REF, False, -1), (gx.APP_SSSP, True, -1),
                                                 (gx.APP_CC, False, -1), (gx.APP_PAGERANK_REF, False, 1 << 20)])
def test_checkpoint_resume_matches_uninterrupted(tmp_path, app, weighted, budget):
    sym = app == gx.APP_CC
    g = gx.rmat_graph(14, 16, seed=31, P=16, symmetric=sym, weight_seed=5 if weighted else None)
    kw = {"source": 0, "weighted": True} if app == gx.APP_SSSP else {}
    n = 20 if app == gx.APP_PAGERANK_REF else 200
    with gx.Engine(cache_budget_bytes=budget) as e:
        e.load(g)
        full = e.run(app, n, checkpoint_every=3, checkpoint_prefix=str(tmp_path / "ck_"), **kw)
        ref_vals = e.values().copy()
        steps = full["iterations"]
        ref_counts = changed(e, 0, steps)
        ck = sorted(int(p.stem[3:]) for p in tmp_path.glob("ck_*.npy"))
        assert ck and all(s % 3 == 0 for s in ck[:-1]) and ck[-1] <= steps
        k = [s for s in ck if 0 < s < steps][-1] if any(0 < s < steps for s in ck) else None
        if k is None:
            pytest.skip("run too short to resume inside it")
        init = gx.read_values(tmp_path / f"ck_{k}.npy", g.V)
        e.set_init(init)
        res = e.run(app, n, use_init=True, first_step=k, **kw)
        assert res["iterations"] == steps
        assert np.array_equal(e.values().view(np.uint32), ref_vals.view(np.uint32))
        assert changed(e, k, steps) == ref_counts[k:]
        assert changed(e, 0, k) == [0] * k
        e.write_values(tmp_path / "final.npy")
        assert np.array_equal(np.load(tmp_path / "final.npy").view(np.uint32), ref_vals.view(np.uint32))


def test_resume_argument_checks():
    g = gx.rmat_graph(10, 8, seed=1, P=4)
    with gx.Engine() as e:
        e.load(g)
        with pytest.raises(gx.GxError):
            e.run(gx.APP_PAGERANK_REF, 10, first_step=3)                 # needs use_init
        with pytest.raises(gx.GxError):
            e.run(gx.APP_PAGERANK_REF, 10, async_mode=True)              # SSSP/CC only
        with pytest.raises(gx.GxError):
            e.run(gx.APP_PAGERANK_REF, 10, checkpoint_every=2)           # needs a prefix


@pytest.mark.parametrize("push", [1, 0])
def test_async_mode_same_fixed_point(push):
    g = gx.rmat_graph(15, 16, seed=7, P=8, weight_seed=99)
    ref, _, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000, weights=g.weights, source=0)
    with gx.Engine(push_sparse=push) as e:
        e.load(g)
        jac = e.run(gx.APP_SSSP, 1000, source=0, weighted=True)
        gs = e.run(gx.APP_SSSP, 1000, source=0, weighted=True, async_mode=True)
        assert np.array_equal(e.values(), ref)
        assert gs["iterations"] <= jac["iterations"]
        ref_u, _, _ = O.run(O.SSSP, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 1000, source=0)
        e.run(gx.APP_SSSP, 1000, source=0, async_mode=True)
        assert np.array_equal(e.values(), ref_u)
    gs_ = gx.rmat_graph(15, 8, seed=12, P=8, symmetric=True)
    ref_cc, _, _ = O.run(O.CC, gs_.V, gs_.P, gs_.bounds, gs_.off, gs_.col, gs_.outdeg, 1000)
    with gx.Engine(push_sparse=push) as e:
        e.load(gs_)
        jac = e.run(gx.APP_CC, 1000)
        gs = e.run(gx.APP_CC, 1000, async_mode=True)
        assert np.array_equal(e.values(), ref_cc)
        assert gs["iterations"] <= jac["iterations"]
