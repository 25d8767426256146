"""FP64 reference of the fusion cost model's network (test infrastructure).

The library trains its MLP with its own CUDA kernels; this numpy restatement
is the checker for their forward pass, loss and gradients.  Parameter layout
(one flat vector): W1 [F x 64] row-major, b1 [64], W2 [64 x 64], b2 [64],
W3 [64 x 64], b3 [64], w4 [64], b4 [1].  Loss: mean of (out - y)^2.
"""
import numpy as np

H = 64


def layout(F: int):
    sizes = [("W1", F * H), ("b1", H), ("W2", H * H), ("b2", H), ("W3", H * H), ("b3", H),
             ("w4", H), ("b4", 1)]
    off, out = 0, {}
    for name, n in sizes:
        out[name] = (off, n)
        off += n
    return out, off


def unpack(p: np.ndarray, F: int):
    lay, _ = layout(F)
    g = {k: p[o:o + n] for k, (o, n) in lay.items()}
    return (g["W1"].reshape(F, H), g["b1"], g["W2"].reshape(H, H), g["b2"],
            g["W3"].reshape(H, H), g["b3"], g["w4"], g["b4"][0])


def forward(p: np.ndarray, x: np.ndarray, F: int) -> np.ndarray:
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p.astype(np.float64), F)
    h1 = np.maximum(x @ W1 + b1, 0)
    h2 = np.maximum(h1 @ W2 + b2, 0)
    h3 = np.maximum(h2 @ W3 + b3, 0)
    return h3 @ w4 + b4


def loss_grad(p: np.ndarray, x: np.ndarray, y: np.ndarray, F: int):
    """(mean squared error, gradient of it w.r.t. the flat parameters)."""
    x = x.astype(np.float64)
    y = y.astype(np.float64)
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p.astype(np.float64), F)
    n = len(y)
    z1 = x @ W1 + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2 + b2
    h2 = np.maximum(z2, 0)
    z3 = h2 @ W3 + b3
    h3 = np.maximum(z3, 0)
    out = h3 @ w4 + b4
    d = 2.0 * (out - y) / n
    g3 = np.outer(d, w4) * (z3 > 0)
    g2 = (g3 @ W3.T) * (z2 > 0)
    g1 = (g2 @ W2.T) * (z1 > 0)
    grads = [x.T @ g1, g1.sum(0), h1.T @ g2, g2.sum(0), h2.T @ g3, g3.sum(0), h3.T @ d,
             np.array([d.sum()])]
    return float(np.mean((out - y) ** 2)), np.concatenate([g.reshape(-1) for g in grads])
