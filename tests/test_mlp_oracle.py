"""Pins the warm-start MLP's FP64 oracle (oracle/gx_mlp_oracle.py), which has
no counterpart in the reference, on CPU:

* its backward pass against torch autograd in FP64 and against central finite
  differences of its own loss;
* its six per-vertex features against an independent scipy.sparse
  restatement (sums as sparse products, the maximum by a loop over lists).

The oracle's forward pass rounds W1, W2 and w3 to BF16 and its gradient is
taken through that rounding as if it were the identity (straight through).
At weights that are already BF16 values the rounding is exact, so there the
oracle's gradient must equal the true gradient of the FP64 network."""
import numpy as np
import pytest

import gx_mlp_oracle as MO

H, F = MO.H, MO.F
N_PARAMS = H * F + H + H * H + H + H + 1


def _bf16_exact_params(rng):
    p = rng.normal(0, 0.3, size=N_PARAMS).astype(np.float32)
    w_slices = [slice(0, H * F), slice(H * F + H, H * F + H + H * H),
                slice(H * F + 2 * H + H * H, H * F + 3 * H + H * H)]
    for s in w_slices:
        p[s] = MO.bf16_round(p[s]).astype(np.float32)
    return p.astype(np.float64)


def _problem(seed, n=200):
    rng = np.random.default_rng(seed)
    p = _bf16_exact_params(rng)
    norm = np.concatenate([rng.normal(0, 1, F), rng.uniform(0.5, 2, F)])
    x = rng.normal(0, 2, size=(n, F))
    t = rng.normal(0, 1.5, size=n)     # some targets above log(100): the weight cap is exercised
    return p, norm, x, t


@pytest.mark.parametrize("seed", [0, 1])
def test_backward_matches_torch_autograd(seed):
    torch = pytest.importorskip("torch")
    p, norm, x, t = _problem(seed)
    loss, g = MO.loss_and_grad(p, norm, x, t)

    pt = torch.tensor(p, dtype=torch.float64, requires_grad=True)
    o = 0
    W1 = pt[o:o + H * F].reshape(H, F); o += H * F
    b1 = pt[o:o + H]; o += H
    W2 = pt[o:o + H * H].reshape(H, H); o += H * H
    b2 = pt[o:o + H]; o += H
    w3 = pt[o:o + H]; o += H
    b3 = pt[o]
    nt = torch.tensor(norm, dtype=torch.float64)
    X = (torch.tensor(x, dtype=torch.float64) - nt[:F]) * nt[F:]
    tt = torch.tensor(t, dtype=torch.float64)
    gelu = torch.nn.functional.gelu
    h1 = gelu(X @ W1.T + b1, approximate="tanh")
    h2 = gelu(h1 @ W2.T + b2, approximate="tanh")
    z = h2 @ w3 + b3
    y = torch.log(torch.nn.functional.softplus(z, beta=1.0, threshold=20.0))
    wt = torch.clamp(torch.exp(tt), max=100.0)
    L = torch.mean(wt * (y - tt) ** 2)
    L.backward()
    ref = pt.grad.numpy()

    assert abs(loss - L.item()) <= 1e-12 * max(1.0, abs(L.item()))
    assert np.abs(g - ref).max() <= 1e-10 * np.abs(ref).max(), np.abs(g - ref).max()


def test_backward_matches_finite_differences_on_biases():
    """Biases are not rounded, so the oracle's own loss can be differentiated
    numerically in them without any other implementation."""
    p, norm, x, t = _problem(3)
    _, g = MO.loss_and_grad(p, norm, x, t)
    rng = np.random.default_rng(4)
    b1_idx = H * F + rng.choice(H, 4, replace=False)
    b2_idx = H * F + H + H * H + rng.choice(H, 4, replace=False)
    idx = np.concatenate([b1_idx, b2_idx, [N_PARAMS - 1]])
    h = 1e-5
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (MO.loss_and_grad(pp, norm, x, t)[0] - MO.loss_and_grad(pm, norm, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1e-3, abs(g[i])), (int(i), fd, g[i])


def test_features_match_sparse_restatement():
    sp = pytest.importorskip("scipy.sparse")
    import graphee_gb300 as gx
    g = gx.rmat_graph(12, 16, seed=21, P=4)
    f = MO.features(g.V, g.off, g.col, g.outdeg)
    off = np.asarray(g.off, np.int64)
    col = np.asarray(g.col, np.int64)
    indeg = np.diff(off).astype(np.float64)
    # A[u, v] = 1 for every edge u -> v: column v of the CSC lists v's sources.
    A = sp.csc_matrix((np.ones(len(col)), col, off), shape=(g.V, g.V))
    lo = np.log1p(np.asarray(g.outdeg, np.float64))
    s = A.T @ lo
    two_hop = A.T @ indeg
    mx = np.array([lo[col[off[v]:off[v + 1]]].max() if off[v + 1] > off[v] else 0.0 for v in range(g.V)])
    np.testing.assert_allclose(f[:, 0], np.log1p(indeg), rtol=0, atol=0)
    np.testing.assert_allclose(f[:, 1], lo, rtol=0, atol=0)
    np.testing.assert_allclose(f[:, 2], np.where(indeg > 0, s / np.maximum(indeg, 1), 0), rtol=1e-14, atol=0)
    np.testing.assert_array_equal(f[:, 3], mx)
    np.testing.assert_allclose(f[:, 4], np.log1p(two_hop), rtol=1e-14, atol=0)
    np.testing.assert_array_equal(f[:, 5], (np.asarray(g.outdeg) == 0).astype(np.float64))
    # the graph has every kind of vertex the features distinguish
    assert (indeg == 0).any() and (np.asarray(g.outdeg) == 0).any() and indeg.max() > 100


def test_forward_is_the_loss_forward():
    """predict() and the loss share one forward pass: targets equal to the
    network's own log-outputs give zero loss and zero gradient."""
    p, norm, x, _ = _problem(5)
    t = np.log(MO.predict(p, norm, x))
    loss, g = MO.loss_and_grad(p, norm, x, t)
    assert loss < 1e-24 and np.abs(g).max() < 1e-12
