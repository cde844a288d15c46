"""pytreegrav_gb300.cuda contexts (pytreegrav.cuda's CudaPotential, CudaAccel, CudaPotentialBruteforce,
CudaAccelBruteforce) against the oracle, following pytreegrav's tests of its CUDA path
(test_cuda_gravity.py:69-122, 142-153, 235-252, 286-304).

The contexts narrow positions and softenings to float32. The oracle therefore gets the same
float32-rounded inputs, widened to float64, and evaluates them in FP64.

Tolerances:
- tree contexts (FP32 walk, per-target opening test, the node set accepted in FP64): 1e-5 relative
  RMS, the bar pytreegrav sets for its FP32 walk;
- brute-force contexts (FP32 direct sums over all sources): 1e-5 relative RMS and 1e-4 relative per
  target. Each target's rounding grows like sqrt(number of sources) x 6e-8; pytreegrav's own test
  scales its tolerance the same way.
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RMS_TOL = 1e-5
MAX_TOL = 1e-4


@pytest.fixture(scope="module")
def cu():
    from pytreegrav_gb300 import cuda

    if not cuda.is_available():
        pytest.skip("needs a CUDA GPU and the built library")
    return cuda


def rel_rms(a, ref):
    a, ref = np.asarray(a, np.float64).reshape(len(a), -1), np.asarray(ref).reshape(len(ref), -1)
    return np.sqrt(np.mean(np.sum((a - ref) ** 2, 1))) / np.sqrt(np.mean(np.sum(ref**2, 1)))


def rel_max(a, ref):
    a, ref = np.asarray(a, np.float64).reshape(len(a), -1), np.asarray(ref).reshape(len(ref), -1)
    scale = np.sqrt(np.mean(np.sum(ref**2, 1)))
    mag = np.maximum(np.sqrt(np.sum(ref**2, 1)), scale)
    return np.max(np.sqrt(np.sum((a - ref) ** 2, 1)) / mag)


def r32(a):
    return np.asarray(a, np.float32).astype(np.float64)


def plummer(n, rng):
    u = rng.random(n)
    r = np.minimum(1 / np.sqrt(u ** (-2 / 3) - 1), 50.0)
    d = rng.normal(size=(n, 3))
    return d / np.linalg.norm(d, axis=1)[:, None] * r[:, None]


def source_set(n=20_000, seed=11):
    rng = np.random.default_rng(seed)
    x = plummer(n, rng)
    m = rng.uniform(0.5, 1.5, n) / n
    h = rng.uniform(0.005, 0.02, n)
    return x, m, h


def oracle_per_target(x, m, h, xt, ht, theta, key):
    """The per-target FP64 walk (group_size 1, pytreegrav's treewalk semantics) on float32-rounded
    inputs, results in the targets' order."""
    res, _ = O.target_fields(r32(xt), r32(ht), r32(x), m, r32(h), potential=key == "potential",
                             accel=key == "accel", theta=theta, group_size=1)
    return res[key]


@pytest.mark.parametrize("key", ["potential", "accel"])
def test_tree_context_matches_per_target_walk(cu, key):
    x, m, h = source_set()
    import pytreegrav_gb300 as tg

    tree = tg.ConstructTree(x, m, h)
    ctx = (cu.CudaPotential if key == "potential" else cu.CudaAccel)(tree)
    rng = np.random.default_rng(3)
    xt = rng.uniform(-3, 3, (3000, 3))
    ht = rng.uniform(0.0, 0.02, 3000)
    got = ctx(xt, ht, G=1.0, theta=0.7)
    assert got.dtype == np.float32
    assert got.shape == ((3000,) if key == "potential" else (3000, 3))
    want = oracle_per_target(x, m, h, xt, ht, 0.7, key)
    assert rel_rms(got, want) < RMS_TOL
    assert rel_max(got, want) < MAX_TOL


def test_tree_context_theta_per_call_and_G(cu):
    """One upload, a different opening angle per call (test_cuda_gravity.py:142-153); G scales."""
    x, m, h = source_set(8000, seed=5)
    import pytreegrav_gb300 as tg

    ctx = cu.CudaAccel(tg.ConstructTree(x, m, h))
    xt = x[:2000]
    for theta in (0.4, 0.7, 1.0):
        got = ctx(xt, h[:2000], G=2.5, theta=theta)
        want = 2.5 * oracle_per_target(x, m, h, xt, h[:2000], theta, "accel")
        assert rel_rms(got, want) < RMS_TOL, theta
    a04, a10 = ctx(xt, h[:2000], theta=0.4), ctx(xt, h[:2000], theta=1.0)
    assert not np.array_equal(a04, a10)


def test_tree_context_drops_self_terms(cu):
    """Targets that are the sources themselves (float64 as given) land on their own float32-rounded
    source, so r == 0 drops the self term (test_target_self_potential.py:23-51; cuda.py:416-418)."""
    x, m, h = source_set(5000, seed=7)
    import pytreegrav_gb300 as tg

    ctx = cu.CudaPotential(tg.ConstructTree(x, m, h))
    got = ctx(x, h)
    want = oracle_per_target(x, m, h, x, h, 0.7, "potential")
    assert rel_rms(got, want) < RMS_TOL
    # a spurious softened self term would add about -2.8 m/h, many times the tolerance
    assert np.max(np.abs(got - want) / np.abs(want)) < MAX_TOL


def test_tree_context_accepts_host_tree_arrays(cu):
    """Any object with pytreegrav's Octree attributes is accepted (the reference takes its jitclass)."""
    x, m, h = source_set(4000, seed=9)
    t = O.OracleTree(x, m, h)

    class HostTree:
        NumParticles = t.NumParticles
        Coordinates = t.Coordinates
        Masses = t.Masses
        Softenings = t.Softenings

    ctx = cu.CudaAccel(HostTree())
    xt = x[::4]
    got = ctx(xt, h[::4])
    want = oracle_per_target(x, m, h, xt, h[::4], 0.7, "accel")
    assert rel_rms(got, want) < RMS_TOL


@pytest.mark.parametrize("key", ["potential", "accel"])
def test_bruteforce_context_targets_and_self(cu, key):
    x, m, h = source_set(6000, seed=13)
    cls = cu.CudaPotentialBruteforce if key == "potential" else cu.CudaAccelBruteforce
    ctx = cls(x, m, h)
    rng = np.random.default_rng(4)
    xt = rng.uniform(-2, 2, (1500, 3))
    ht = rng.uniform(0.0, 0.01, 1500)
    got = ctx(xt, ht, G=3.0)
    assert got.dtype == np.float32
    want = O.bruteforce(r32(xt), r32(ht), r32(x), r32(m), r32(h), potential=key == "potential",
                        accel=key == "accel", G=3.0)[key]
    assert rel_rms(got, want) < RMS_TOL
    assert rel_max(got, want) < MAX_TOL
    # pos=None: the sources themselves, self term excluded (distinct points: index and r == 0 agree)
    got_self = ctx()
    want_self = O.bruteforce(r32(x), r32(h), r32(x), r32(m), r32(h), potential=key == "potential",
                             accel=key == "accel", mutual=True)[key]
    assert got_self.shape == want_self.shape
    assert rel_rms(got_self, want_self) < RMS_TOL
    assert rel_max(got_self, want_self) < MAX_TOL


def test_bruteforce_context_scalar_softening_and_reuse(cu):
    x, m, _ = source_set(3000, seed=17)
    ctx = cu.CudaAccelBruteforce(x, m, 0.01)
    for seed in range(3):  # repeated calls against the same upload
        xt = np.random.default_rng(seed).normal(size=(700, 3))
        got = ctx(xt, 0.002)
        want = O.bruteforce(r32(xt), r32(np.full(700, 0.002)), r32(x), r32(m), r32(np.full(3000, 0.01)),
                            accel=True)["accel"]
        assert rel_rms(got, want) < RMS_TOL
