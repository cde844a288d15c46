"""Node velocities and the two-point functions on the GPU (tg_tree_set_velocities, tg_tree_correlation).

* Velocities and dispersions of every node equal the oracle's ComputeMomentsDynamic restatement on
  the same tree bit for bit (the same chain order and the same roundings, no contraction).
* Each kind (density, velocity correlation, structure function) x binning (weighted, jittered by the
  shared counter-based generator, every particle on its own) x geometry (open, periodic box) x
  targets (the tree's own particles, other points): GPU bin sums against the oracle's within 1e-12 of
  the per-bin sum of absolute contributions -- the summation order over targets differs, nothing else.
* The frontends end to end against pytreegrav's own outputs (tests/golden/golden_corr.npz) at the
  same relative bar (1e-12 of the bin's absolute scale from the oracle).
* A larger case (2e5 Plummer particles, theta 1 and 0.5) through the same comparison, and edge
  cases: no targets, a single bin, a tree without velocities asked for a velocity function.
* The walk decides in FP32 when a decision is clear of its threshold and falls back to pytreegrav's
  FP64 expression otherwise: a periodic lattice whose offsets are exactly half the box exercises the
  fallback, against the oracle at the same bar.
"""

import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def tg():
    import pytreegrav_gb300 as tg

    return tg


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_corr.npz"))


def plummer_with_flow(n, seed):
    from pytreegrav_gb300 import synthetic

    x = synthetic.plummer(n, seed)
    rng = np.random.default_rng(seed + 1)
    m = rng.random(n) / n
    v = 0.3 * x + rng.normal(size=(n, 3))
    return x, m, v


def compare(gpu, ora, absum, kind):
    (b, w), (bo, wo) = gpu, ora
    assert np.all(np.abs(b - bo) <= TOL * np.maximum(absum, 1e-300)), (kind, np.max(np.abs(b - bo) / np.maximum(absum, 1e-300)))
    if kind != "density":
        assert np.all(np.abs(w - wo) <= TOL * np.maximum(wo, 1e-300))


@pytest.fixture(scope="module")
def trees(tg):
    x, m, v = plummer_with_flow(20_000, 31)
    t = tg.ConstructTree(x, m, np.zeros(len(x)), vel=v)
    ot = O.OracleTree(x, m, np.zeros(len(x)))
    return x, m, v, t, ot, O.tree_velocities(ot, v)


def test_node_velocities_bit_exact(trees):
    x, m, v, t, ot, (ov, od) = trees
    assert t.HasVelocities
    nh = t.node_hi
    assert np.array_equal(t.Velocities[:nh], ov[:nh])
    assert np.array_equal(t.VelocityDisp[:nh], od[:nh])
    assert np.all(t.Velocities[nh:] == 0) and np.all(t.VelocityDisp[nh:] == 0)
    assert t.Velocities.shape == (t.NumNodes, 3)


@pytest.mark.parametrize("kind", ["density", "velocity", "structure"])
@pytest.mark.parametrize("binning", ["weighted", "jitter", "pairs"])
@pytest.mark.parametrize("box", [0.0, 6.0])
@pytest.mark.parametrize("own", [True, False])
def test_correlation_vs_oracle(trees, kind, binning, box, own):
    x, m, v, t, ot, otv = trees
    rb = 10 ** np.linspace(-2.0, 0.6, 17)
    kw = dict(theta=0.8, boxsize=box, max_bin_size_ratio=100.0)
    if binning == "weighted":
        kw["weighted_binning"] = True
    elif binning == "pairs":
        kw["max_bin_size_ratio"] = 1e-300
    seed = 1234
    idx = ot.TreewalkIndices
    if own:
        pos, vel, wt = x[idx], v[idx], m[idx]
        gpu = t.correlation(kind, None, rb, seed=seed, **kw)
    else:
        rng = np.random.default_rng(5)
        pos = rng.normal(size=(3_000, 3))
        vel = rng.normal(size=(3_000, 3))
        wt = rng.random(3_000)
        gpu = t.correlation(kind, pos, rb, vel=vel, weight=wt, seed=seed, **kw)
    extra = {} if kind == "density" else dict(vel=vel, weight=wt, tree_vel=otv)
    ora = O.correlation(ot, kind, pos, rb, seed=seed, nthreads=O.num_threads(), **extra, **kw)
    absum, _ = O.correlation(ot, kind, pos, rb, seed=seed, absval=True, nthreads=O.num_threads(), **extra, **kw)
    compare(gpu, ora, absum, kind)


def test_frontends_match_pytreegrav(tg, g):
    x, m, v = g["pos"], g["m"], g["v"]
    n = len(x)
    ot = O.OracleTree(x, m, np.zeros(n))
    otv = O.tree_velocities(ot, v)
    idx = ot.TreewalkIndices
    rb = g["rbins"]

    def scale(kind, r, **kw):
        extra = {} if kind == "density" else dict(vel=v[idx], weight=m[idx], tree_vel=otv)
        a, w = O.correlation(ot, kind, x[idx], r, absval=True, theta=kw.pop("theta", 1.0), **extra, **kw)
        return a / n if kind == "density" else a / w

    r0, got = tg.DensityCorrFunc(x, m, weighted_binning=True)
    assert np.array_equal(r0, g["rbins_default"])
    assert np.all(np.abs(got - g["density_weighted"]) <= TOL * scale("density", r0, weighted_binning=True))
    for name, fn, kind, kw in [
        ("density_pairs", tg.DensityCorrFunc, "density", dict(max_bin_size_ratio=1e-300)),
        ("density_weighted_t0.5", tg.DensityCorrFunc, "density", dict(theta=0.5, weighted_binning=True)),
        ("velocity_weighted", tg.VelocityCorrFunc, "velocity", dict(weighted_binning=True)),
        ("velocity_pairs", tg.VelocityCorrFunc, "velocity", dict(max_bin_size_ratio=1e-300)),
        ("structure_weighted", tg.VelocityStructFunc, "structure", dict(weighted_binning=True)),
        ("structure_weighted_t0.6_mbr3", tg.VelocityStructFunc, "structure",
         dict(theta=0.6, max_bin_size_ratio=3.0, weighted_binning=True)),
    ]:
        args = (x, m) if kind == "density" else (x, m, v)
        _, got = fn(*args, rb, **kw)
        ref = g[name]
        assert np.array_equal(np.isfinite(got), np.isfinite(ref)), name
        ok = np.isfinite(ref)
        assert np.all(np.abs(got[ok] - ref[ok]) <= TOL * scale(kind, rb, **kw)[ok]), name
    # periodic box
    xu, mu, vu, rb3 = g["box/pos"], g["box/m"], g["box/v"], g["box/rbins"]
    _, got = tg.DensityCorrFunc(xu, mu, rb3, boxsize=1.0, weighted_binning=True)
    assert np.allclose(got, g["box/density_weighted"], rtol=1e-12, atol=0)
    _, got = tg.VelocityStructFunc(xu, mu, vu, rb3, boxsize=1.0, weighted_binning=True)
    assert np.allclose(got, g["box/structure_weighted"], rtol=1e-12, atol=0)
    # a supplied tree and other targets (Morton-ordered by the frontend); return_tree
    tree = tg.ConstructTree(x, m, np.zeros(n))
    _, got, t2 = tg.DensityCorrFunc(g["targets/pos"], np.ones(150), rb, tree=tree, weighted_binning=True,
                                    return_tree=True)
    assert t2 is tree
    assert np.allclose(got, g["targets/density_weighted"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("theta", [1.0, 0.5])
def test_larger_case(tg, theta):
    x, m, v = plummer_with_flow(200_000, 37)
    _, _, t = tg.VelocityStructFunc(x, m, v, 10 ** np.linspace(-2.5, 1, 24), theta=theta, return_tree=True, seed=9)
    ot = O.OracleTree(x, m, np.zeros(len(x)))
    otv = O.tree_velocities(ot, v)
    idx = ot.TreewalkIndices
    rb = 10 ** np.linspace(-2.5, 1, 24)
    for kind in ("density", "velocity", "structure"):
        for wb in (True, False):
            kw = dict(theta=theta, weighted_binning=wb, seed=9)
            gpu = t.correlation(kind, None, rb, **kw)
            extra = {} if kind == "density" else dict(vel=v[idx], weight=m[idx], tree_vel=otv)
            ora = O.correlation(ot, kind, x[idx], rb, nthreads=O.num_threads(), **extra, **kw)
            a, _ = O.correlation(ot, kind, x[idx], rb, absval=True, nthreads=O.num_threads(), **extra, **kw)
            compare(gpu, ora, a, kind)


def test_edge_cases(tg):
    x, m, v = plummer_with_flow(2_000, 41)
    t = tg.ConstructTree(x, m, None, vel=v)
    rb = np.array([0.01, 10.0])  # one bin
    b, w = t.correlation("structure", None, rb, weighted_binning=True)
    assert b.shape == (1,) and w[0] > 0
    b, w = t.correlation("density", np.zeros((0, 3)), rb)
    assert np.all(b == 0)
    plain = tg.ConstructTree(x, m)
    with pytest.raises(ValueError):
        plain.correlation("velocity", None, rb)
    with pytest.raises(ValueError):
        tg.VelocityCorrFunc(x[:10], m[:10], v[:10], rb, tree=plain)
    with pytest.raises(ValueError):
        t.correlation("density", None, np.array([1.0]))


@pytest.mark.parametrize("kind", ["density", "velocity", "structure"])
def test_screen_fallbacks_periodic_lattice(tg, kind):
    """A lattice of spacing box/8 in a periodic box: many offsets are exactly half the box (the FP32
    screen cannot decide the nearest image there and the FP64 expression does) and many distances are
    equal. GPU sums against the oracle's at the same bar, jittered and weighted."""
    g = np.arange(8) * 0.25
    x = np.ascontiguousarray(np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3))
    n = len(x)
    rng = np.random.default_rng(9)
    m = rng.random(n) / n
    v = rng.normal(size=(n, 3))
    t = tg.ConstructTree(x, m, None, vel=v)
    ot = O.OracleTree(x, m, np.zeros(n))
    otv = O.tree_velocities(ot, v)
    idx = ot.TreewalkIndices
    rb = 10 ** np.linspace(-0.93, 0.07, 7)  # edges away from the lattice's distances
    for wb in (False, True):
        kw = dict(theta=0.9, boxsize=2.0, weighted_binning=wb, seed=77)
        gpu = t.correlation(kind, None, rb, **kw)
        extra = {} if kind == "density" else dict(vel=v[idx], weight=m[idx], tree_vel=otv)
        ora = O.correlation(ot, kind, x[idx], rb, **extra, **kw)
        a, _ = O.correlation(ot, kind, x[idx], rb, absval=True, **extra, **kw)
        compare(gpu, ora, a, kind)
