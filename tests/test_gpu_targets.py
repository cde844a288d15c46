"""External targets grouped by their own octree (TargetSet, tg_targets_*), plain and learned.

* The grouping: groups partition the targets in the target tree's walk order, each of at most
  group_size targets, and the walk-order permutation is a permutation.
* Plain walks of those groups against the oracle walking the same groups (fields_groups with the
  set's own starts and counts): FP64 to summation-order rounding (1e-12), FP32 at the walk bar
  (1e-5 relative RMS, 1e-4 max).
* The learned acceptance test for external targets, on a reduced form of the largest configuration
  (Plummer sources with lognormal softenings, uniform targets in a ball of radius 5): judged by FP64
  brute force on every target, its RMS force error stays within 1.15x the plain theta = 0.7 walk's
  on the same groups, with fewer interactions.
* The frontend: AccelTarget / PotentialTarget with grouping="tree" or learned=True equal the
  TargetSet calls; with the default grouping they stay pytreegrav's (oracle target_fields).
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP32_RMS, FP32_MAX, FP64_TOL = 1e-5, 1e-4, 1e-12


@pytest.fixture(scope="module")
def tg():
    import pytreegrav_gb300 as tg

    return tg


def rel_rms(a, ref):
    a, ref = np.asarray(a).reshape(len(a), -1), np.asarray(ref).reshape(len(ref), -1)
    return np.sqrt(np.mean(np.sum((a - ref) ** 2, 1))) / np.sqrt(np.mean(np.sum(ref**2, 1)))


def rel_max(a, ref):
    a, ref = np.asarray(a).reshape(len(a), -1), np.asarray(ref).reshape(len(ref), -1)
    scale = np.sqrt(np.mean(np.sum(ref**2, 1)))
    mag = np.maximum(np.sqrt(np.sum(ref**2, 1)), scale)
    return np.max(np.sqrt(np.sum((a - ref) ** 2, 1)) / mag)


def sources(n, seed, lognormal_h=True):
    """Plummer sources with float32-rounded positions, masses 1/n, softenings lognormal
    (mu = ln 0.003, sigma = 0.7) or 0.005."""
    from pytreegrav_gb300 import synthetic

    x = synthetic.plummer(n, seed).astype(np.float32).astype(np.float64)
    rng = np.random.default_rng(seed + 1)
    h = np.exp(rng.normal(np.log(0.003), 0.7, n)) if lognormal_h else np.full(n, 0.005)
    return x, np.full(n, 1.0 / n), h


def ball_targets(n, seed, radius=5.0):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    return d * (radius * rng.random(n) ** (1 / 3))[:, None]


@pytest.mark.parametrize("gs", [8, 32])
def test_target_groups_partition(tg, gs):
    x, m, h = sources(20_000, 3)
    xt = ball_targets(7_001, 4)
    tree = tg.ConstructTree(x, m, h, quadrupole=True)
    ts = tg.TargetSet(tree, xt, np.zeros(len(xt)), group_size=gs)
    first, count, node, widx = ts.groups()
    assert np.all(count >= 1) and np.all(count <= gs)
    assert first[0] == 0 and np.all(first[1:] == first[:-1] + count[:-1]) and first[-1] + count[-1] == len(xt)
    assert np.array_equal(np.sort(widx), np.arange(len(xt)))
    assert np.all(node >= 0) and np.all(node < tree.node_hi - tree.NumParticles)
    # each group's source node is a cell holding the group's box: the box fits in the cell's size
    xs = xt[widx]
    sizes = tree.Sizes[tree.NumParticles + node]
    for g in range(0, len(first), max(1, len(first) // 200)):
        b = xs[first[g]:first[g] + count[g]]
        assert np.all(b.max(0) - b.min(0) <= sizes[g] * (1 + 1e-12))


@pytest.mark.parametrize("quad", [False, True])
def test_target_set_walk_vs_oracle(tg, quad):
    x, m, h = sources(60_000, 5, lognormal_h=True)
    xt = ball_targets(20_000, 6)
    ht = np.full(len(xt), 0.002)
    tree = tg.ConstructTree(x, m, h, quadrupole=True)
    ot = O.OracleTree(x, m, h, quadrupole=True)
    ts = tg.TargetSet(tree, xt, ht, group_size=32)
    first, count, _, widx = ts.groups()
    ref_w = O.fields_groups(ot, xt[widx], ht[widx], first, count, True, True, True, quad, 0.7,
                            nthreads=O.num_threads())
    for prec, tol, mtol in (("fp64", FP64_TOL, FP64_TOL), ("fp32", FP32_RMS, FP32_MAX)):
        got = ts.fields(True, True, True, quadrupole=quad, theta=0.7, precision=prec)
        for k in got:
            ref = np.empty_like(ref_w[k])
            ref[widx] = ref_w[k]
            assert rel_rms(got[k], ref) < tol, (prec, k, rel_rms(got[k], ref))
            assert rel_max(got[k], ref) < mtol, (prec, k, rel_max(got[k], ref))
    # the frontend's grouping="tree" is the same walk
    a = tg.AccelTarget(xt, x, m, ht, h, theta=0.7, quadrupole=quad, method="tree", grouping="tree", group_size=32)
    assert np.array_equal(a, ts.fields(accel=True, quadrupole=quad, theta=0.7)["accel"])


def test_target_default_grouping_is_pytreegrav(tg):
    """Without the extension keywords the target forms keep pytreegrav's blocks of group_size."""
    x, m, h = sources(30_000, 7, lognormal_h=False)
    xt = ball_targets(5_000, 8)
    ref, _ = O.target_fields(xt, None, x, m, h, accel=True, potential=True, theta=0.7, quadrupole=True,
                             nthreads=O.num_threads())
    a = tg.AccelTarget(xt, x, m, None, h, theta=0.7, quadrupole=True, method="tree")
    p = tg.PotentialTarget(xt, x, m, None, h, theta=0.7, quadrupole=True, method="tree")
    assert rel_rms(a, ref["accel"]) < FP32_RMS and rel_max(a, ref["accel"]) < FP32_MAX
    assert rel_rms(p, ref["potential"]) < FP32_RMS


def test_learned_targets_reduced_largest(tg):
    """1e6 Plummer sources (lognormal softenings), 1e5 uniform targets in r < 5: the learned test for
    external targets against FP64 brute force over all sources, next to plain theta = 0.7 on the same
    target groups."""
    x, m, h = sources(1_000_000, 9)
    xt = ball_targets(100_000, 10)
    ht = np.zeros(len(xt))
    tree = tg.ConstructTree(x, m, h, quadrupole=True)
    ts = tg.TargetSet(tree, xt, ht, group_size=32)
    ref = tg.bruteforce(xt, ht, x, m, h, accel=True, potential=True, precision="fp64")
    plain = ts.fields(accel=True, potential=True, quadrupole=True, theta=0.7)
    n_plain = tree.last_walk_stats()[0]
    learned = ts.fields_learned(accel=True, potential=True, quadrupole=True, theta=0.7)
    n_learned = tree.last_walk_stats()[0]
    e_plain, e_learned = rel_rms(plain["accel"], ref["accel"]), rel_rms(learned["accel"], ref["accel"])
    print(f"\nreduced largest configuration: plain RMS {e_plain:.2e} ({n_plain / len(xt):.0f} interactions/target), "
          f"learned RMS {e_learned:.2e} ({n_learned / len(xt):.0f}); max {rel_max(learned['accel'], ref['accel']):.2e}")
    assert e_learned < 1.15 * e_plain
    assert n_learned < n_plain
    # the frontend call is the same walk
    a = tg.AccelTarget(xt, None, None, ht, tree=tree, theta=0.7, quadrupole=True, method="tree", learned=True)
    assert np.array_equal(a, ts.fields_learned(accel=True, quadrupole=True, theta=0.7)["accel"])


def test_target_set_edge_cases(tg):
    x, m, h = sources(5_000, 12, lognormal_h=False)
    tree = tg.ConstructTree(x, m, h, quadrupole=True)
    # one target; targets on top of sources (r == 0 pairs skipped); all targets at one point
    for xt in (x[:1], x[:257], np.repeat(x[:1], 100, axis=0)):
        ht = np.full(len(xt), 0.005)
        ts = tg.TargetSet(tree, xt, ht, group_size=32)
        got = ts.fields(potential=True, accel=True, quadrupole=True, theta=0.7)
        ref, _ = O.target_fields(xt, ht, x, m, h, potential=True, accel=True, theta=0.7, quadrupole=True,
                                 tree=O.OracleTree(x, m, h, quadrupole=True))
        for k in got:  # different grouping: the accepted sets differ, both close to the exact field
            assert np.all(np.isfinite(got[k]))
            assert rel_rms(got[k], ref[k]) < 5e-3
    with pytest.raises(RuntimeError):
        bad = np.array(x[:10])
        bad[3, 1] = np.nan
        tg.TargetSet(tree, bad)
