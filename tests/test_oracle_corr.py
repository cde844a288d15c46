"""The oracle's two-point functions against pytreegrav's own (tests/golden/golden_corr.npz).

* DynamicOctree: pytreegrav's insertion-built velocity tree (dynamic_tree.py) visits the particles in
  the radix tree's walk order and has the same nodes in the same traversal order; node masses,
  centres, Deltas, velocities and dispersions agree with the oracle's radix tree and
  ComputeMomentsDynamic restatement to rounding (the two builds add children's masses in different
  orders), sizes exactly.
* DensityCorrFunc / VelocityCorrFunc / VelocityStructFunc in their deterministic forms (weighted
  binning; or every particle binned on its own): each bin within 1e-13 of the sum of the absolute
  values of its contributions (the oracle with absval) -- rounding, since the summation order over
  targets differs.
* The default rbins heuristic, the periodic box, and targets that are not the tree's particles.
* The jitter generator: uniform on [0, 1), and the jittered density conserves the mass that the
  weighted form bins, away from the range's ends.
"""

import numpy as np
import pytest

from oracle import oracle as O

TOL = 1e-13


@pytest.fixture(scope="module")
def g():
    import os

    return np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_corr.npz"))


@pytest.fixture(scope="module")
def setup(g):
    x, m, v = g["pos"], g["m"], g["v"]
    t = O.OracleTree(x, m, np.zeros(len(x)))
    return x, m, v, t, O.tree_velocities(t, v)


def preorder(t, tv):
    n = t.NumParticles
    order, nodes, st = [], [], [n]
    while st:
        no = st.pop()
        if no < n:
            order.append(no)
            continue
        nodes.append(np.concatenate([[t.Masses[no]], t.Coordinates[no], [t.Sizes[no], t.Deltas[no]], tv[0][no],
                                     [tv[1][no]]]))
        kids, c, stop = [], t.FirstSubnode[no], t.NextBranch[no]
        while c != -1 and c != stop:
            kids.append(c)
            c = t.NextBranch[c]
        st.extend(reversed(kids))
    return np.array(order), np.array(nodes)


def test_dynamic_octree_is_the_radix_tree(g, setup):
    x, m, v, t, tv = setup
    order, nodes = preorder(t, tv)
    # same particles visited in the same order, same nodes in the same traversal order
    assert np.array_equal(t.TreewalkIndices[order], g["dyn/TreewalkIndices"][g["dyn/order"]])
    ref = g["dyn/nodes_preorder"]
    assert nodes.shape == ref.shape
    assert np.array_equal(nodes[:, 4], ref[:, 4])  # sizes
    scale = np.abs(ref).max(0)
    assert np.all(np.abs(nodes - ref).max(0) <= 1e-14 * np.maximum(scale, 1.0))
    # the root's velocity is the mass-weighted mean, its dispersion the mass-weighted variance about it
    root = t.NumParticles
    vm = (m[:, None] * v).sum(0) / m.sum()
    assert np.allclose(tv[0][root], vm, rtol=1e-12, atol=1e-14)
    assert np.isclose(tv[1][root], (m * ((v - vm) ** 2).sum(1)).sum() / m.sum(), rtol=1e-12)
    assert np.all(tv[1][: t.NumParticles] == 0)


def _check(t, tv, kind, pos, vel, wt, rbins, ref, n, **kw):
    extra = {} if kind == "density" else dict(vel=vel, weight=wt, tree_vel=tv)
    b, w = O.correlation(t, kind, pos, rbins, **extra, **kw)
    a, _ = O.correlation(t, kind, pos, rbins, absval=True, **extra, **kw)
    if kind == "density":
        err = np.abs(b / n - ref) / np.maximum(a / n, 1e-300)
    else:
        ok = w > 0
        assert np.array_equal(ok, np.isfinite(ref))
        err = np.abs(b[ok] - ref[ok] * w[ok]) / np.maximum(a[ok], 1e-300)
    assert err.max() < TOL, (kind, kw, err.max())
    return b, w


CASES = [
    ("density_weighted", "density", dict(weighted_binning=True), "rbins_default"),
    ("density_pairs", "density", dict(max_bin_size_ratio=1e-300), "rbins"),
    ("density_weighted_t0.5", "density", dict(theta=0.5, weighted_binning=True), "rbins"),
    ("velocity_weighted", "velocity", dict(weighted_binning=True), "rbins"),
    ("velocity_pairs", "velocity", dict(max_bin_size_ratio=1e-300), "rbins"),
    ("structure_weighted", "structure", dict(weighted_binning=True), "rbins"),
    ("structure_weighted_t0.6_mbr3", "structure", dict(theta=0.6, max_bin_size_ratio=3.0, weighted_binning=True),
     "rbins"),
]


@pytest.mark.parametrize("name,kind,kw,rb", CASES, ids=[c[0] for c in CASES])
def test_correlation_matches_pytreegrav(g, setup, name, kind, kw, rb):
    x, m, v, t, tv = setup
    idx = t.TreewalkIndices  # the frontend's target order for a tree it builds
    kw = dict(kw)
    kw.setdefault("theta", 1.0)
    _check(t, tv, kind, x[idx], v[idx], m[idx], g[rb], g[name], len(x), **kw)


def test_default_rbins_heuristic(g):
    from pytreegrav_gb300.frontend import _default_rbins

    assert np.array_equal(_default_rbins(g["pos"]), g["rbins_default"])


def test_periodic_box(g):
    xu, mu, vu, rb = g["box/pos"], g["box/m"], g["box/v"], g["box/rbins"]
    t = O.OracleTree(xu, mu, np.zeros(len(xu)))
    tv = O.tree_velocities(t, vu)
    i = t.TreewalkIndices
    _check(t, tv, "density", xu[i], None, None, rb, g["box/density_weighted"], len(xu), theta=1.0, boxsize=1.0,
           weighted_binning=True)
    _check(t, tv, "structure", xu[i], vu[i], mu[i], rb, g["box/structure_weighted"], len(xu), theta=1.0, boxsize=1.0,
           weighted_binning=True)


def test_targets_other_than_the_tree(g, setup):
    x, m, v, t, tv = setup
    xt = g["targets/pos"]
    o = O.morton_order(xt)
    _check(t, tv, "density", xt[o], None, None, g["rbins"], g["targets/density_weighted"], len(xt), theta=1.0,
           weighted_binning=True)


def test_jitter_generator_and_mass_conservation(g, setup):
    u = np.array([O.corr_uniform(5, i, d) for i in range(200) for d in range(20)])
    assert u.min() >= 0 and u.max() < 1 and abs(u.mean() - 0.5) < 0.01 and abs(u.var() - 1 / 12) < 0.003
    assert O.corr_uniform(5, 3, 4) != O.corr_uniform(6, 3, 4) != O.corr_uniform(5, 4, 4)
    x, m, v, t, tv = setup
    idx = t.TreewalkIndices
    rb = g["rbins"]
    jit, _ = O.correlation(t, "density", x[idx], rb, theta=1.0, seed=11)
    wgt, _ = O.correlation(t, "density", x[idx], rb, theta=1.0, weighted_binning=True)
    # both bin each accepted node's whole mass once; only the bins it lands in differ
    assert np.isclose(jit[2:-2].sum(), wgt[2:-2].sum(), rtol=0.05)
    again, _ = O.correlation(t, "density", x[idx], rb, theta=1.0, seed=11)
    assert np.array_equal(jit, again)
