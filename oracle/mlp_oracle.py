"""FP64 restatement of the cost model's forward and backward pass.

Test infrastructure only: checks the gradients computed by the library's
own CUDA kernels (btc_mlp_gradient).  Network: n_in -> 32 -> 32 -> 1 with
tanh hidden units; loss = mean squared error; weights flat as
W1[32][n_in], b1[32], W2[32][32], b2[32], w3[32], b3.
"""
import numpy as np

H = 32


def unpack(p, n_in):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * n_in].reshape(H, n_in); o += H * n_in
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, x):
    W1, b1, W2, b2, w3, b3 = unpack(p, x.shape[1])
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ w3 + b3, h1, h2


def gradient(p, x, t):
    """(flat gradient, loss) of mean((y - t)^2)."""
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    n = len(t)
    W1, b1, W2, b2, w3, b3 = unpack(p, x.shape[1])
    y, h1, h2 = forward(p, x)
    e = y - t
    dy = 2.0 * e / n
    g_w3 = h2.T @ dy
    g_b3 = dy.sum()
    dz2 = (dy[:, None] * w3[None, :]) * (1 - h2 ** 2)
    g_W2 = dz2.T @ h1
    g_b2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * (1 - h1 ** 2)
    g_W1 = dz1.T @ x
    g_b1 = dz1.sum(0)
    g = np.concatenate([g_W1.ravel(), g_b1, g_W2.ravel(), g_b2, g_w3, [g_b3]])
    return g, float((e ** 2).mean())
