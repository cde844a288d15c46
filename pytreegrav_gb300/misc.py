"""Host helpers with pytreegrav.misc's names."""

import numpy as np


def random_rotation(seed):
    """A random rotation matrix, reproducible from `seed` (misc.py:7-55): a uniform random x axis,
    a second random axis orthogonalised against it and normalised, z their cross product. Draws
    from numpy's legacy generator seeded with `seed`, as pytreegrav does, but from a private
    RandomState, so the global numpy generator is left alone."""
    rs = np.random.RandomState(seed)
    R = np.zeros((3, 3))
    for row in range(2):
        costheta = rs.uniform(-1, 1)
        sintheta = np.sqrt(max(1 - costheta * costheta, 0))
        phi = 2 * np.pi * rs.uniform(0, 1)
        R[row] = sintheta * np.cos(phi), sintheta * np.sin(phi), costheta
    s = 0
    for k in range(3):
        s += R[0, k] * R[1, k]
    for k in range(3):
        R[1, k] -= s * R[0, k]
    s = 0
    for k in range(3):
        s += R[1, k] * R[1, k]
    s = np.sqrt(s)
    for k in range(3):
        R[1, k] /= s
    for i in range(3):
        j, k = (i + 1) % 3, (i + 2) % 3
        R[2, i] = R[0, j] * R[1, k] - R[1, j] * R[0, k]
    return R
