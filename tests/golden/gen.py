"""Platform-independent synthetic particle sets for fixtures.

numpy's Generator streams and libm's transcendental functions may differ in the last bit between
numpy versions and between x86 and Arm, which would break bit-exact digests of a tree built from
them. These inputs use splitmix64 integers and only +, -, *, / and sqrt -- operations IEEE 754
rounds identically everywhere -- so the same seed gives the same doubles on every machine.
"""

import numpy as np

_M64 = (1 << 64) - 1


def splitmix64(seed, n):
    """n successive splitmix64 outputs as uint64 (vectorised; wraps modulo 2^64)."""
    with np.errstate(over="ignore"):
        s = np.uint64(seed & _M64) + np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
        z = s
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed, n):
    """n doubles in [0, 1) from the top 53 bits."""
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def concentrated(seed, n):
    """n points in a centrally concentrated cloud: a uniform ball point q scaled by |q|^2.

    Density rises steeply towards the centre (like a cusp), which gives deep trees; only exact
    arithmetic and sqrt are used.
    """
    out = np.empty((0, 3))
    k = 0
    while len(out) < n:
        u = uniform(seed + 7919 * k, 3 * 2 * n).reshape(-1, 3) * 2.0 - 1.0
        r2 = u[:, 0] * u[:, 0] + u[:, 1] * u[:, 1] + u[:, 2] * u[:, 2]
        u = u[(r2 < 1.0) & (r2 > 0.0)]
        out = np.vstack([out, u])
        k += 1
    q = out[:n]
    r2 = q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1] + q[:, 2] * q[:, 2]
    return q * r2[:, None] * 4.0


def masses(seed, n):
    return (uniform(seed, n) + 0.5) / n


def softenings(seed, n, hmax):
    return uniform(seed, n) * hmax
