"""Seeded synthetic particle systems: the distributions the benchmarks and the opening-angle
training use (no dataset ships with pytreegrav's benchmarks either)."""

import numpy as np


def plummer(n, seed, a=1.0, rmax=50.0):
    """Plummer sphere of scale a, radii r = a / sqrt(u^(-2/3) - 1) truncated at r < rmax,
    isotropic directions."""
    rng = np.random.default_rng(seed)
    out = np.empty((0, 3))
    while len(out) < n:
        k = n - len(out)
        u = rng.random(k)
        r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        d = rng.normal(size=(k, 3))
        p = d / np.linalg.norm(d, axis=1)[:, None] * r[:, None]
        out = np.vstack([out, p[r < rmax * a]])
    return np.ascontiguousarray(out[:n])


def clustered(n, seed, k=64, box=20.0):
    """Mixture of k Plummer subclusters: centres uniform in a cube of side `box`, scale radii
    lognormal (mu = ln 0.3, sigma = 0.5), member counts multinomial with Dirichlet(1) weights."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-box / 2, box / 2, (k, 3))
    radii = np.exp(rng.normal(np.log(0.3), 0.5, k))
    counts = rng.multinomial(n, rng.dirichlet(np.ones(k)))
    parts = [plummer(c, int(rng.integers(1 << 31)), a=rc) + ctr
             for c, rc, ctr in zip(counts, radii, centres) if c > 0]
    out = np.vstack(parts)
    return np.ascontiguousarray(out[rng.permutation(len(out))])


def uniform(n, seed):
    """Uniform in the unit cube."""
    return np.random.default_rng(seed).random((n, 3))
