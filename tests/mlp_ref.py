"""numpy restatement of the opening-angle network and its training kernels (test checker only):
16-64-64-1 with SiLU, the flat parameter layout of include/pytreegrav_gb300_theta.h, the
interpolated cost/error loss and Adam."""

import numpy as np

NF, H = 16, 64
NP = H * NF + H + H * H + H + H + 1


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * NF].reshape(H, NF); o += H * NF
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sigmoid(z)


def dsilu(z):
    s = sigmoid(z)
    return s * (1.0 + z * (1.0 - s))


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    z1 = x @ W1.T + b1
    z2 = silu(z1) @ W2.T + b2
    y = silu(z2) @ W3 + b3
    return y, z1, z2


def backward(p, x, dy):
    """Gradient of sum(dy * y) with respect to the flat parameters."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    _, z1, z2 = forward(p, x)
    dz2 = dy[:, None] * W3[None, :] * dsilu(z2)
    dz1 = (dz2 @ W2) * dsilu(z1)
    g = np.concatenate([(dz1.T @ x).ravel(), dz1.sum(0), (dz2.T @ silu(z1)).ravel(), dz2.sum(0),
                        (dy[:, None] * silu(z2)).sum(0), [dy.sum()]])
    return g


def theta_loss(y, lc, le, lam, t0, dt, tmin, tmax):
    """(mean loss, d loss / d y) of the interpolated cost + lambda * error loss."""
    n, K = lc.shape
    s = sigmoid(y)
    th = tmin + (tmax - tmin) * s
    u = (th - t0) / dt
    k = np.clip(np.floor(u).astype(int), 0, K - 2)
    w = u - k
    r = np.arange(n)
    logc = lc[r, k] + w * (lc[r, k + 1] - lc[r, k])
    loge = le[r, k] + w * (le[r, k + 1] - le[r, k])
    cost, err = np.exp(logc), np.exp(loge)
    loss = cost + lam * err
    dl = (cost * (lc[r, k + 1] - lc[r, k]) + lam * err * (le[r, k + 1] - le[r, k])) / dt
    dy = dl * (tmax - tmin) * s * (1 - s) / n
    return loss.mean(), dy


def adam(p, g, m, v, lr, b1, b2, eps, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v
