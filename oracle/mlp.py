"""FP64 NumPy restatement of the rank predictor's network -- TEST INFRASTRUCTURE ONLY.

8 -> 64 -> 64 -> 1 with ReLU, loss 0.5 * mean((f(x) - y)^2), parameters laid out
as the library stores them (W1 64x8, b1, W2 64x64, b2, W3 1x64, b3, row-major,
concatenated) and features standardised with (x - mean) / std. Used only to
check the library's forward and backward kernels.
"""
import numpy as np

IN, H = 8, 64
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (1, H)), ("b3", (1,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, off = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[off:off + n], np.float64).reshape(shape)
        off += n
    return out


def forward(p, norm, X):
    w = unpack(p)
    Z = (np.asarray(X, np.float64) - norm[:IN]) / norm[IN:]
    A1 = Z @ w["W1"].T + w["b1"]
    H1 = np.maximum(A1, 0)
    A2 = H1 @ w["W2"].T + w["b2"]
    H2 = np.maximum(A2, 0)
    out = H2 @ w["W3"].T + w["b3"]
    return out[:, 0], (Z, A1, H1, A2, H2)


def loss_and_grad(p, norm, X, y):
    w = unpack(p)
    out, (Z, A1, H1, A2, H2) = forward(p, norm, X)
    n = len(y)
    e = out - np.asarray(y, np.float64)
    loss = 0.5 * np.mean(e ** 2)
    g_out = e / n
    gW3 = g_out @ H2
    gb3 = g_out.sum()
    d2 = np.outer(g_out, w["W3"][0]) * (A2 > 0)
    gW2 = d2.T @ H1
    gb2 = d2.sum(0)
    d1 = (d2 @ w["W2"]) * (A1 > 0)
    gW1 = d1.T @ Z
    gb1 = d1.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), [gb3]])
    return loss, grad
