"""FP64 restatement of the warm-start MLP (forward, loss, backward) and of
its input features.

TEST INFRASTRUCTURE ONLY: the correctness reference for the GPU training kernels'
gradients and the feature kernel.  Same parameter layout as the library:
W1[64][6], b1[64], W2[64][64], b2[64], w3[64], b3; forward uses W1, W2, w3
rounded to BF16 (round to nearest even), biases in full precision.
"""
import numpy as np

H, F = 64, 6


def bf16_round(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * F].reshape(H, F); o += H * F
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


C_GELU = np.sqrt(2 / np.pi)


def gelu(x):
    """GELU in its tanh form, as the library computes it."""
    return 0.5 * x * (1 + np.tanh(C_GELU * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C_GELU * (x + 0.044715 * x ** 3))
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * C_GELU * (1 + 3 * 0.044715 * x * x)


def softplus(z):
    return np.where(z > 20, z, np.log1p(np.exp(np.minimum(z, 20))))


def predict(params, norm, x_raw):
    """softplus(z) of the network in FP64, with W1, W2, w3 rounded to BF16
    as the library's forward passes use them (before normalisation to sum 1)."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    p32 = np.asarray(params, np.float32)
    W1r = bf16_round(p32[:H * F]).reshape(H, F)
    W2r = bf16_round(p32[H * F + H:H * F + H + H * H]).reshape(H, H)
    w3r = bf16_round(p32[H * F + 2 * H + H * H:H * F + 3 * H + H * H])
    norm = np.asarray(norm, np.float64)
    X = (np.asarray(x_raw, np.float64) - norm[:F]) * norm[F:]
    return softplus(gelu(gelu(X @ W1r.T + b1) @ W2r.T + b2) @ w3r + b3)


def loss_and_grad(params, norm, x_raw, t):
    """Mean over samples of min(exp(t), 100) * (log softplus(z) - t)^2 and its gradient."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    p32 = np.asarray(params, np.float32)
    W1r = bf16_round(p32[:H * F]).reshape(H, F)
    W2r = bf16_round(p32[H * F + H:H * F + H + H * H]).reshape(H, H)
    w3r = bf16_round(p32[H * F + 2 * H + H * H:H * F + 3 * H + H * H])
    norm = np.asarray(norm, np.float64)
    X = (np.asarray(x_raw, np.float64) - norm[:F]) * norm[F:]
    t = np.asarray(t, np.float64)
    n = len(t)
    A1 = X @ W1r.T + b1
    H1 = gelu(A1)
    A2 = H1 @ W2r.T + b2
    H2 = gelu(A2)
    z = H2 @ w3r + b3
    sp = softplus(z)
    y = np.log(sp)
    e = y - t
    wt = np.minimum(np.exp(t), 100.0)
    loss = np.mean(wt * e * e)
    dz = 2 * wt * e / n * (1 / (1 + np.exp(-z))) / sp
    g_w3 = H2.T @ dz
    g_b3 = dz.sum()
    D2 = dz[:, None] * w3r[None, :] * gelu_grad(A2)
    g_W2 = D2.T @ H1
    g_b2 = D2.sum(0)
    D1 = (D2 @ W2r) * gelu_grad(A1)
    g_W1 = D1.T @ X
    g_b1 = D1.sum(0)
    g = np.concatenate([g_W1.ravel(), g_b1, g_W2.ravel(), g_b2, g_w3, [g_b3]])
    return loss, g


def features(V, off, col, outdeg):
    """The six per-vertex features, in FP64."""
    off = np.asarray(off, np.int64)
    col = np.asarray(col, np.int64)
    indeg = np.diff(off)
    lo = np.log1p(np.asarray(outdeg, np.float64))
    dst = np.repeat(np.arange(V), indeg)
    s = np.zeros(V)
    np.add.at(s, dst, lo[col])
    mx = np.zeros(V)
    np.maximum.at(mx, dst, lo[col])
    s2 = np.zeros(V)
    np.add.at(s2, dst, indeg[col].astype(np.float64))
    f = np.zeros((V, F))
    f[:, 0] = np.log1p(indeg)
    f[:, 1] = lo
    f[:, 2] = np.where(indeg > 0, s / np.maximum(indeg, 1), 0)
    f[:, 3] = mx
    f[:, 4] = np.log1p(s2)
    f[:, 5] = (np.asarray(outdeg) == 0).astype(np.float64)
    return f
