"""Bounded device-side waits, driven to their limit without faulting or
hanging the GPU: the CTA-team barrier of the batched kernel and the grid
barrier of the persistent PPR launch poll at most config.wait_limit times;
with a limit of one poll a barrier gives up, every CTA leaves through the
abort flag, and the call returns GX_ERR_TIMEOUT.  The same engine then runs
again with the normal limit and matches the oracle."""
import numpy as np
import pytest

import graphee_gb300 as gx
import gx_oracle as O

pytestmark = pytest.mark.gpu


def _instance(g, vb, i):
    b, e = int(vb[i]), int(vb[i + 1])
    off = g.off[b:e + 1] - g.off[b]
    col = g.col[g.off[b]:g.off[e]] - b
    return e - b, off, col, g.outdeg[b:e]


def test_team_barrier_timeout_then_recovery():
    # 48 instances, scales 8..17: the largest get CTA teams (several CTAs
    # that meet at a global barrier after every superstep).
    g, vb = gx.batch_graph(48, scales=(8, 17), edge_factors=(8, 16), seed=11)
    with gx.Engine() as e:
        e.load(g)
        e.set_wait_limit(1)
        with pytest.raises(gx.GxError) as ei:
            e.batch_run(vb, pr_iters=30, cc_max_iter=1000)
        assert ei.value.status == gx.GX_ERR_TIMEOUT
        e.set_wait_limit(1 << 24)
        pr, cc, ps, cs, st = e.batch_run(vb, pr_iters=30, cc_max_iter=1000)
    big = int(np.argmax(np.diff(g.off[vb])))
    for i in (big, 0):
        n, off, col, od = _instance(g, vb, i)
        b = np.array([0, n], np.int32)
        ref, ch, _ = O.run(O.PAGERANK_REF, n, 1, b, off, col, od, 30)
        sl = slice(vb[i], vb[i + 1])
        assert np.abs(pr[sl] - ref).max() / ref.max() < 1e-5, i
        assert ps[i] == len(ch)
        lab, chc, _ = O.run(O.CC, n, 1, b, off, col, od, 1000)
        assert np.array_equal(cc[sl], lab) and cs[i] == len(chc), i


def test_wait_limit_must_be_positive():
    with pytest.raises(gx.GxError) as ei:
        gx.Engine(wait_limit=0)
    assert ei.value.status == gx.GX_ERR_INVALID
    with gx.Engine() as e:
        with pytest.raises(gx.GxError):
            e.set_wait_limit(0)


def test_ppr_grid_barrier_timeout_then_recovery():
    g = gx.rmat_graph(15, 16, seed=8, P=4)
    src = np.array([0, 5, 77, 1000], np.int32)
    with gx.Engine() as e:
        e.load(g)
        e.set_wait_limit(1)
        with pytest.raises(gx.GxError) as ei:
            e.ppr(src, 10)
        assert ei.value.status == gx.GX_ERR_TIMEOUT
        e.set_wait_limit(1 << 24)
        R, st = e.ppr(src, 10)
    ref = O.ppr(g.V, g.off, g.col, g.outdeg, src, 10, 0.15)
    assert np.abs(R - ref).max() < 1e-6
