"""Column density on the GPU (tg_tree_column_density, ColumnDensity, CudaColumnDensity) against
pytreegrav's own walks and a direct sum, following pytreegrav's test_column_density.py.

Tolerances:
- against the golden fixtures (pytreegrav's Python walks on the same tree) and the oracle: zero,
  because the GPU walks are FP64 in the reference's order of operations, each operation rounded once;
- against direct summation: 1e-12 relative to the largest column, pytreegrav's own bar. The
  ray-traced walk has no truncation error, only rounding.
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-12
SIX_RAYS = np.vstack([np.eye(3), -np.eye(3)])


@pytest.fixture(scope="module")
def tg():
    import pytreegrav_gb300 as tg

    return tg


def column_direct(pos_target, rays, x, m, h):
    """Direct sum over all sources of the uniform-sphere chord (numpy, no tree); (Nt, Nr)."""
    d = x[None, :, :] - pos_target[:, None, :]
    r2 = (d * d).sum(-1)
    z = np.einsum("tsk,rk->tsr", d, rays)
    b2 = np.maximum(r2[:, :, None] - z * z, 0.0)
    hs = np.where(h > 0, h, 1.0)
    fac = np.where(h > 0, 3 * m / (4 * np.pi * hs**2), 0.0)[None, :, None]
    chord = np.sqrt(np.maximum(1 - b2 / (hs * hs)[None, :, None], 0.0))
    hits = (b2 < (h * h)[None, :, None]) & (h > 0)[None, :, None]
    outside = (r2 > (h * h)[None, :])[:, :, None]
    full = hits & outside & (z > 0)
    partial = hits & ~outside
    contrib = np.where(full, fac * 2 * chord, 0.0) + np.where(partial, fac * (z / hs[None, :, None] + chord), 0.0)
    return contrib.sum(1)


def cloud(n, seed=42, scale=3.0):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 3))
    return x, np.ones(n) / n, np.full(n, scale * n ** (-1 / 3))


def rel(a, b):
    s = np.abs(b).max()
    return np.abs(a - b).max() / (s if s > 0 else 1.0)


def test_walks_equal_pytreegrav_and_oracle(tg, golden_column):
    g = golden_column
    t = tg.ConstructTree(g["src/pos"], g["src/m"], g["src/h"])
    got = t.column_density(g["tgt/pos"], g["rays"])
    assert np.array_equal(got, g["rays_out"])
    for theta in (0.5, 0.8):
        assert np.array_equal(t.column_density(g["tgt/pos"], None, theta), g[f"binned_theta{theta}"])
    per = np.ascontiguousarray(np.broadcast_to(g["rays"], (len(g["tgt/pos"]),) + g["rays"].shape))
    assert np.array_equal(t.column_density(g["tgt/pos"], per), g["rays_out"])
    for gs in (1, 7, 16):  # the grouped binned walk
        assert np.array_equal(t.column_density(g["grouped/pos"], None, 0.5, gs), g[f"binned_grouped_gs{gs}"]), gs


@pytest.mark.parametrize("n", [500, 4000])
def test_ray_traced_matches_direct_sum(tg, n):
    x, m, h = cloud(n)
    rng = np.random.default_rng(3)
    rays = rng.normal(size=(5, 3))
    rays /= np.linalg.norm(rays, axis=1)[:, None]
    rays = np.vstack([SIX_RAYS, rays])
    cols = tg.ColumnDensity(x, m, h, rays=rays)
    assert rel(cols, column_direct(x, rays, x, m, h)) < RTOL
    # external targets, prebuilt tree of the same particles
    xt = rng.normal(size=(300, 3)) * 2
    t = tg.ConstructTree(x, m, h)
    assert rel(tg.ColumnDensity(xt, m[:300], h[:300], rays=rays, tree=t), column_direct(xt, rays, x, m, h)) < RTOL


def test_wide_radius_range_and_zero_radii(tg):
    rng = np.random.default_rng(5)
    n = 2000
    x = rng.normal(size=(n, 3))
    m = rng.random(n) / n
    h = 10 ** rng.uniform(-3, 0, n)
    h[::17] = 0.0  # point-like: no cross-section
    with pytest.warns(UserWarning, match="radii are <= 0"):
        cols = tg.ColumnDensity(x, m, h, rays=6)
    assert np.all(np.isfinite(cols))
    assert rel(cols, column_direct(x, SIX_RAYS, x, m, h)) < RTOL
    with pytest.warns(UserWarning):
        assert np.all(tg.ColumnDensity(x, m, np.zeros(n), rays=6) == 0)


def test_frontend_matches_the_oracle_in_the_callers_order(tg):
    x, m, h = cloud(3000, seed=9)
    ot = O.OracleTree(x, m, h)
    idx = ot.TreewalkIndices
    rays = SIX_RAYS
    ref_sorted = O.column_rays(ot, x[idx], rays)
    ref = np.empty_like(ref_sorted)
    ref[idx] = ref_sorted
    cols, tree = tg.ColumnDensity(x, m, h, rays=6, return_tree=True)
    assert np.array_equal(cols, ref)
    # 3000 targets: pytreegrav groups the binned walk (16 consecutive Morton targets by default)
    binned_sorted = O.column_binned_grouped(ot, x[idx], 0.5, 16)
    binned = np.empty_like(binned_sorted)
    binned[idx] = binned_sorted
    assert np.array_equal(tg.ColumnDensity(x, m, h), binned)
    small = O.column_binned(ot, x[idx][:500], 0.5)  # below 1000 targets: the per-target walk
    assert np.array_equal(tg.ColumnDensity(x[idx][:500], m[:500], h[:500], tree=tree), small)
    with pytest.raises(ValueError, match="group_size"):
        tg.ColumnDensity(x, m, h, group_size=64)
    assert np.array_equal(tg.ColumnDensity(x, m, h, tree=tree, rays=6), ref)


def test_randomize_rays_rotates_each_grid_by_its_morton_position(tg):
    from pytreegrav_gb300.misc import random_rotation

    x, m, h = cloud(800, seed=11)
    ot = O.OracleTree(x, m, h)
    idx = ot.TreewalkIndices
    per = np.array([SIX_RAYS @ random_rotation(i) for i in range(len(x))])
    ref_sorted = O.column_rays(ot, x[idx], per, per_target=True)
    ref = np.empty_like(ref_sorted)
    ref[idx] = ref_sorted
    assert np.array_equal(tg.ColumnDensity(x, m, h, rays=6, randomize_rays=True), ref)
    # each target's own rotated rays against the direct sum
    direct = np.array([column_direct(x[idx][i:i + 1], per[i], x, m, h)[0] for i in range(0, len(x), 97)])
    assert rel(ref_sorted[::97], direct) < RTOL


def test_binned_estimator_conserves_mass_far_away(tg):
    """A target far from the cloud sees the whole mass in one bin as a point mass at the centre of mass
    (the whole tree is accepted): column = M / r^2 / (4 pi / 6)."""
    x, m, h = cloud(1000, seed=13, scale=0.5)
    far = np.array([[1e4, 0.0, 0.0]])
    t = tg.ConstructTree(x, m, h)
    col = t.column_density(far, None, 0.5)[0]
    com = (m[:, None] * x).sum(0) / m.sum()
    r2 = ((com - far[0]) ** 2).sum()
    assert col[1] == pytest.approx(m.sum() / r2 / (4 * np.pi / 6), rel=1e-9)
    assert np.count_nonzero(col) == 1


def test_cuda_context_is_reusable_and_float32(tg):
    from pytreegrav_gb300 import cuda

    if not cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    x, m, h = cloud(2000, seed=15)
    t = tg.ConstructTree(x, m, h)
    ctx = cuda.CudaColumnDensity(t)
    rays = np.array([[2.0, 0.0, 0.0], [0.0, 0.0, -3.0]])  # normalised by the context
    a = ctx(x, rays)
    b = ctx(x, rays)
    assert a.dtype == np.float32 and a.shape == (2000, 2)
    assert np.array_equal(a, b)
    unit = rays / np.linalg.norm(rays, axis=1)[:, None]
    assert np.array_equal(a, t.column_density(x, unit).astype(np.float32))
    one = ctx(x[:5], [0.0, 1.0, 0.0])  # a single ray
    assert one.shape == (5, 1)
    with pytest.raises(ValueError, match="ray-traced path"):
        tg.ColumnDensity(x, m, h, rays=None, device="cuda")
    dev = tg.ColumnDensity(x, m, h, rays=6, device="cuda")
    assert dev.dtype == np.float32


def test_own_particles_form_equals_the_explicit_targets(tg):
    """tg_tree_column_density with pos NULL walks the tree's own particles in walk order and writes
    each row at its caller index: the same numbers as the explicit Morton-ordered targets, unsorted."""
    x, m, h = cloud(3000, seed=17)
    t = tg.ConstructTree(x, m, h)
    idx = t.TreewalkIndices
    xs = x[idx]
    rng = np.random.default_rng(4)
    per = rng.normal(size=(len(x), 4, 3))
    per /= np.linalg.norm(per, axis=2)[:, :, None]
    for args in ((SIX_RAYS,), (per,), (None, 0.5, 0), (None, 0.7, 16)):
        explicit = t.column_density(xs, *args)
        unsorted = np.empty_like(explicit)
        unsorted[idx] = explicit
        assert np.array_equal(t.column_density_self(*args), unsorted)
