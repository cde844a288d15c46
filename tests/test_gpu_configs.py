"""The benchmark configurations run as written, on the GPU, through the public API.

* Uniform cube, N = 1e5 (float64, seeded), m = 1/N, h = 0.01, theta = 0.7, monopole: Accel and
  Potential via method='tree' against method='bruteforce' on a 1e4-target subset (the reference's
  tree_test.py bar, 0.02, is far looser than what the tree gives here; the bars below are ~2x the
  oracle's own errors on this input, so a broken walk fails them).
* Plummer sphere, N = 1e6 (a = 1, r < 50), m = 1/N, h = 0.005, quadrupole, theta in {0.4, 0.7}:
  Accel, Potential and the tidal tensor with pytreegrav's default grouping (8 consecutive Morton
  targets), FP32 walk with FP64 tree; (1) against the oracle walking the same groups, at the FP32 walk
  bar (1e-5 relative RMS), and (2) against FP64 brute force on 1e4 sampled targets, normalised as
  examples/error_benchmark.py:74-76 does (rms|a|, std(phi) after removing the mean offset, rms|T|),
  with bars set from the oracle's errors on the same input (measured on the CPU: theta = 0.7 ->
  accel 7.9e-4, potential 1.5e-4, tidal 8.0e-4; theta = 0.4 -> 6.8e-5, 1.6e-5, 7.3e-5).
* Clustered mixture, N = 4e6 (64 Plummer subclusters), h = 0.002, quadrupole: the learned acceptance
  test judged by FP64 brute force on 1e4 sampled targets: RMS force error at most 1e-3, and no more
  than the plain theta = 0.7 walk's with fewer interactions.
Every result's RMS and max error is printed (pytest -s shows them).
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP32_RMS = 1e-5


@pytest.fixture(scope="module")
def tg():
    import pytreegrav_gb300 as tg

    return tg


def errs(a, ref):
    """(RMS, max) of the per-target error norm, relative to the RMS norm of the reference."""
    a, ref = np.asarray(a).reshape(len(a), -1), np.asarray(ref).reshape(len(ref), -1)
    d = np.sqrt(np.sum((a - ref) ** 2, 1))
    s = np.sqrt(np.mean(np.sum(ref**2, 1)))
    return float(np.sqrt(np.mean(d**2)) / s), float(d.max() / s)


def pot_errs(p, ref):
    """Potential error with the zero point removed, relative to std(phi) (error_benchmark.py:88-91)."""
    d = (p - ref) - np.mean(p - ref)
    return float(np.std(p - ref) / np.std(ref)), float(np.abs(d).max() / np.std(ref))


def plummer(n, seed):
    from pytreegrav_gb300 import synthetic

    return synthetic.plummer(n, seed)


def test_uniform_1e5_tree_vs_bruteforce(tg):
    rng = np.random.default_rng(0)
    n = 100_000
    x = rng.random((n, 3))
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.01)
    a = tg.Accel(x, m, h, theta=0.7, method="tree")
    p = tg.Potential(x, m, h, theta=0.7, method="tree")
    sub = np.random.default_rng(1).choice(n, 10_000, replace=False)
    a_bf = tg.AccelTarget(x[sub], x, m, h[sub], h, method="bruteforce")
    p_bf = tg.PotentialTarget(x[sub], x, m, h[sub], h, method="bruteforce")
    ea, pa = errs(a[sub], a_bf), pot_errs(p[sub], p_bf)
    print(f"\nuniform 1e5, theta 0.7, monopole: accel RMS {ea[0]:.2e} max {ea[1]:.2e}; "
          f"potential RMS {pa[0]:.2e} max {pa[1]:.2e}")
    # the oracle's errors on this input: accel 2.03e-3 (max 6.7e-3), potential 1.05e-3
    assert ea[0] < 3e-3 and ea[1] < 1.5e-2
    assert pa[0] < 2e-3
    # the reference's own bar (tree_test.py): absolute RMS force and potential error < 0.02
    assert np.sqrt(np.mean(np.sum((a[sub] - a_bf) ** 2, 1))) < 0.02
    assert np.std(p[sub] - p_bf) < 0.02


@pytest.fixture(scope="module")
def plummer_1e6(tg):
    n = 1_000_000
    x = plummer(n, 20261203)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.005)
    sub = np.random.default_rng(7).choice(n, 10_000, replace=False)
    bf = tg.bruteforce(x[sub], h[sub], x, m, h, potential=True, accel=True, tidal=True, precision="fp64")
    field = tg.Field(x, m, h, quadrupole=True)
    return x, m, h, sub, bf, field


# bars: about 1.3x the oracle's errors against FP64 brute force on this input (RMS), 2x (max)
BARS = {0.7: dict(accel=1.05e-3, potential=2.0e-4, tidal=1.05e-3),
        0.4: dict(accel=9e-5, potential=2.2e-5, tidal=1.0e-4)}


@pytest.mark.parametrize("theta", [0.4, 0.7])
def test_plummer_1e6_precision_form(tg, plummer_1e6, theta):
    x, m, h, sub, bf, field = plummer_1e6
    n = len(x)
    got = field.evaluate(potential=True, accel=True, tidal=True, theta=theta)  # group_size=8, blocks
    ea, ep, et = errs(got["accel"][sub], bf["accel"]), pot_errs(got["potential"][sub], bf["potential"]), \
        errs(got["tidal"][sub], bf["tidal"])
    print(f"\nPlummer 1e6, theta {theta}, quadrupole, FP32 walk vs FP64 brute force (1e4 targets): "
          f"accel RMS {ea[0]:.2e} max {ea[1]:.2e}; potential RMS {ep[0]:.2e} max {ep[1]:.2e}; "
          f"tidal RMS {et[0]:.2e} max {et[1]:.2e}")
    b = BARS[theta]
    assert ea[0] < b["accel"], ea
    assert ep[0] < b["potential"], ep
    assert et[0] < b["tidal"], et

    # the oracle walking the same groups of 8 (those holding 2000 of the sampled targets)
    ot = O.OracleTree(x, m, h, quadrupole=True)
    idx = ot.TreewalkIndices
    inv = np.empty(n, np.int64)
    inv[idx] = np.arange(n)
    pos_s = inv[sub[:2000]]
    starts = np.unique(pos_s // 8 * 8)
    counts = np.minimum(8, n - starts)
    ref = O.fields_groups(ot, x[idx], h[idx], starts, counts, True, True, True, True, theta,
                          nthreads=O.num_threads())
    for k in ("potential", "accel", "tidal"):
        r = errs(got[k][idx[pos_s]], ref[k][pos_s])
        assert r[0] < FP32_RMS, (k, r)


def test_plummer_1e6_tree_grouping_accuracy(tg, plummer_1e6):
    """The engine's tree grouping (groups of <= 32) at theta = 0.7 against FP64 brute force: the
    accepted set differs from pytreegrav's groups of 8, so the bar is the accuracy itself."""
    x, m, h, sub, bf, field = plummer_1e6
    got = field.tree.fields(potential=True, accel=True, tidal=True, quadrupole=True, group_size=32, theta=0.7,
                            grouping="tree")
    ea, ep, et = errs(got["accel"][sub], bf["accel"]), pot_errs(got["potential"][sub], bf["potential"]), \
        errs(got["tidal"][sub], bf["tidal"])
    print(f"\nPlummer 1e6, theta 0.7, tree grouping 32: accel RMS {ea[0]:.2e} max {ea[1]:.2e}; "
          f"potential RMS {ep[0]:.2e}; tidal RMS {et[0]:.2e}")
    assert ea[0] < 1.05e-3 and ep[0] < 2e-4 and et[0] < 1.05e-3


def test_clustered_4e6_learned(tg):
    """The learned acceptance test on the 4e6-particle clustered mixture (quadrupole, h = 0.002):
    RMS force error <= 1e-3 against FP64 brute force on 1e4 sampled targets, no worse than the
    plain theta = 0.7 walk's, at fewer interactions."""
    from pytreegrav_gb300 import synthetic

    n = 4_000_000
    x = synthetic.clustered(n, 20261204)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.002)
    sub = np.random.default_rng(11).choice(n, 10_000, replace=False)
    ref = tg.bruteforce(x[sub], h[sub], x, m, h, accel=True, precision="fp64")["accel"]
    tree = tg.ConstructTree(x, m, h, quadrupole=True)
    learned = tree.fields(accel=True, quadrupole=True, theta=0.7, learned=True)["accel"]
    n_learned = tree.last_walk_stats()[0]
    plain = tree.fields(accel=True, quadrupole=True, theta=0.7, group_size=32, grouping="tree")["accel"]
    n_plain = tree.last_walk_stats()[0]
    el, ep = errs(learned[sub], ref), errs(plain[sub], ref)
    print(f"\nclustered 4e6: learned RMS {el[0]:.2e} max {el[1]:.2e} ({n_learned / n:.0f} interactions/target); "
          f"plain theta 0.7 RMS {ep[0]:.2e} max {ep[1]:.2e} ({n_plain / n:.0f})")
    assert el[0] <= 1e-3
    assert el[0] <= 1.05 * ep[0]
    assert n_learned < 0.8 * n_plain
