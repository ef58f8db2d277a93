"""CPU FP64 restatement of the learned load balancer's MLP (test
infrastructure: only tests, smoke() and the bench's CPU leg use it).

The model has no reference counterpart; this restatement pins the GPU's
forward pass and gradients.  It mirrors the device's rounding points: the
weights used by the forward pass and the stored activations H1, dH2, dH1 are
rounded to bf16 (round to nearest even); everything else is exact FP64.
With rounding=False it is the plain FP64 network, whose gradient the tests
check against central finite differences.

Parameter layout (one flat float vector): W1 [D][256], b1 [256],
W2 [256 out][256 in], b2 [256], w3 [256], b3 [1], with D = (N-1)*N + 1:
one-hot feature (t-1)*N + cell for each tile t = 1..N-1, then the slack.
"""
import numpy as np

H = 256


def feature_dim(width):
    n = width * width
    return (n - 1) * n + 1


def num_params(width):
    d = feature_dim(width)
    return d * H + H + H * H + H + H + 1


def split(p, width):
    d = feature_dim(width)
    o = 0
    W1 = p[o:o + d * H].reshape(d, H); o += d * H
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o:o + 1]
    return W1, b1, W2, b2, w3, b3


def bf16(x):
    """Round to bf16 (nearest even) via float32, returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def features(tiles, width):
    """Feature indices [n][N-1] of the one-hot part."""
    t = np.asarray(tiles, dtype=np.int64)
    n = width * width
    out = np.empty((t.shape[0], n - 1), dtype=np.int64)
    cells = np.argsort(t, axis=1)  # cells[:, v] = cell of tile v
    for v in range(1, n):
        out[:, v - 1] = (v - 1) * n + cells[:, v]
    return out


def forward_backward(p, tiles, slack, target, width, rounding=True):
    """Loss (mean squared error), prediction y and the flat gradient."""
    p = np.asarray(p, dtype=np.float64)
    W1, b1, W2, b2, w3, b3 = split(p, width)
    r = bf16 if rounding else (lambda x: np.asarray(x, dtype=np.float64))
    W1b, W2b = r(W1), r(W2)
    f = features(tiles, width)
    s = np.asarray(slack, dtype=np.float64)
    t = np.asarray(target, dtype=np.float64)
    nb = f.shape[0]
    d = feature_dim(width)
    z1 = b1[None, :] + s[:, None] * W1b[d - 1][None, :] + W1b[f].sum(axis=1)
    H1 = r(np.maximum(z1, 0.0))
    z2 = H1 @ W2b.T + b2[None, :]
    h2 = np.maximum(z2, 0.0)
    y = h2 @ w3 + b3[0]
    diff = y - t
    loss = float(np.mean(diff * diff))
    dy = 2.0 * diff / nb
    gb3 = np.array([dy.sum()])
    gw3 = h2.T @ dy
    dH2 = dy[:, None] * w3[None, :] * (z2 > 0)
    gb2 = dH2.sum(axis=0)
    dH2b = r(dH2)
    gW2 = dH2b.T @ H1
    dZ1 = dH2b @ W2b
    dH1 = dZ1 * (H1 > 0)
    gb1 = dH1.sum(axis=0)
    dH1b = r(dH1)
    gW1 = np.zeros_like(W1)
    np.add.at(gW1, f.reshape(-1), np.repeat(dH1b, f.shape[1], axis=0))
    gW1[d - 1] += s @ dH1b
    grad = np.concatenate([gW1.reshape(-1), gb1, gW2.reshape(-1), gb2, gw3, gb3])
    return loss, y, grad


def predict(p, tiles, slack, width):
    _, y, _ = forward_backward(p, tiles, slack, np.zeros(len(slack)), width)
    return y
