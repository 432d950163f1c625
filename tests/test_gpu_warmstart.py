"""Learned warm start: the GPU training kernels' gradients against the FP64
oracle, the feature kernel against its FP64 restatement, and what the
trained network gains over the uniform start on a held-out graph."""
import numpy as np
import pytest

import graphee_gb300 as gx
import gx_mlp_oracle as MO
import gx_oracle as O

pytestmark = pytest.mark.gpu


def test_gradient_matches_fp64_oracle():
    m = gx.MLP(seed=5)
    rng = np.random.default_rng(0)
    p, _ = m.params()
    p = p + rng.normal(0, 0.05, size=p.shape).astype(np.float32)   # non-trivial biases
    norm = np.concatenate([rng.normal(0, 1, 6), rng.uniform(0.5, 2, 6)]).astype(np.float32)
    m.set_params(p, norm)
    x = rng.normal(0, 2, size=(300, 6)).astype(np.float32)
    t = rng.normal(0, 1, size=300).astype(np.float32)
    g, loss = m.grad(x, t)
    ref_loss, ref_g = MO.loss_and_grad(p, norm, x, t)
    assert abs(loss - ref_loss) <= 1e-4 * max(1.0, abs(ref_loss))
    scale = np.abs(ref_g).max()
    assert np.abs(g - ref_g).max() <= 2e-4 * scale, np.abs(g - ref_g).max() / scale
    # and the gradient is a descent direction
    assert float(np.dot(g, ref_g)) > 0.99 * np.linalg.norm(g) * np.linalg.norm(ref_g)


def test_inference_matches_fp64_forward():
    """The tensor-core inference (f16 operands and activations, FP32
    accumulation) against the FP64 forward pass of the same network on the
    oracle's features, after normalisation to sum 1."""
    g = gx.rmat_graph(14, 16, seed=11, P=4)
    m = gx.MLP(seed=6)
    p, _ = m.params()
    rng = np.random.default_rng(2)
    p = (p + rng.normal(0, 0.05, size=p.shape)).astype(np.float32)
    F = MO.features(g.V, g.off, g.col, g.outdeg)
    norm = np.concatenate([F.mean(0), 1.0 / (F.std(0) + 1e-6)]).astype(np.float32)
    m.set_params(p, norm)
    with gx.Engine() as e:
        e.load(g)
        pred, _ = m.predict(e)
    ref = MO.predict(p, norm, F)
    ref = ref / ref.sum()
    pred = pred.astype(np.float64)
    l1 = np.abs(pred - ref).sum()
    rel = (np.abs(pred - ref) / ref).max()
    print(f"inference vs FP64 forward: L1 {l1:.2e}, max relative {rel:.2e}")
    assert l1 < 5e-3 and rel < 3e-2, (l1, rel)


def test_prediction_is_normalised_and_training_reduces_loss():
    graphs = [gx.rmat_graph(s, 16, seed=100 + i, P=4) for i, s in enumerate([11, 12, 12, 13])]
    m = gx.MLP(seed=1)
    for g in graphs:
        with gx.Engine() as e:
            e.load(g)
            m.add_graph(e, max_samples=8192)
    l0 = m.train(1, batch=2048, lr=0.0)
    l1 = m.train(30, batch=2048, lr=3e-3)
    assert l1 < 0.5 * l0
    with gx.Engine() as e:
        e.load(graphs[0])
        pred, ms = m.predict(e)
    assert abs(float(pred.astype(np.float64).sum()) - 1.0) < 1e-4 and (pred > 0).all()


def test_warm_start_gains_on_held_out_graph():
    train = [gx.rmat_graph(s, 16, seed=200 + i, P=4, a=0.57 + d, b=0.19 - d / 2, c=0.19 - d / 2)
             for i, (s, d) in enumerate([(12, 0.0), (12, 0.03), (13, -0.03), (13, 0.0), (14, 0.02), (14, -0.02)])]
    m = gx.MLP(seed=3)
    for g in train:
        with gx.Engine() as e:
            e.load(g)
            m.add_graph(e, max_samples=16384)
    m.train(40, batch=4096, lr=3e-3)
    test = gx.rmat_graph(15, 16, seed=999, P=8)
    ref, _, _ = O.run(O.PAGERANK_STD, test.V, test.P, test.bounds, test.off, test.col, test.outdeg, 300,
                      tolerance=1e-12)
    with gx.Engine() as e:
        e.load(test)
        pred, _ = m.predict(e)
        err_warm = np.abs(pred - ref).sum()
        err_unif = np.abs(1.0 / test.V - ref).sum()
        uni = e.run(gx.APP_PAGERANK_STD, 500, tolerance=1e-6)
        ws = e.pagerank_warm(m, 500, tolerance=1e-6)
        vals = e.values().astype(np.float64)
    assert err_warm < 0.5 * err_unif, (err_warm, err_unif)
    assert ws["used_warm"] == 1
    assert ws["resid_warm_first"] < ws["resid_uniform_first"]
    assert ws["iterations"] <= uni["iterations"]
    assert np.abs(vals - ref).sum() < 1e-5


def test_bad_network_falls_back_to_uniform():
    g = gx.rmat_graph(13, 16, seed=7, P=4)
    m = gx.MLP(seed=4)
    p, norm = m.params()
    rng = np.random.default_rng(1)
    m.set_params((rng.normal(0, 3, size=p.shape)).astype(np.float32), norm)
    ref, _, _ = O.run(O.PAGERANK_STD, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 300, tolerance=1e-12)
    with gx.Engine() as e:
        e.load(g)
        ws = e.pagerank_warm(m, 500, tolerance=1e-6)
        vals = e.values().astype(np.float64)
    assert ws["used_warm"] == 0 and ws["resid_warm_first"] > ws["resid_uniform_first"]
    assert np.abs(vals - ref).sum() < 1e-5
