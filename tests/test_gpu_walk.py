"""GPU grouped walk and brute force vs the oracle and the golden fixtures.

Tolerances: the FP64 walk evaluates the reference's accepted node set in double precision, so it
agrees with the oracle to summation-order rounding (1e-12 relative). The FP32 walk (the engine's
default) evaluates the same accepted set in single precision with compensated accumulation: it is
held to 1e-5 relative RMS against the FP64 walk and 1e-4 relative max per target. FP64 brute force
is the reference's arithmetic in the reference's order: bit-exact.
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP32_RMS = 1e-5
FP32_MAX = 1e-4
FP64_TOL = 1e-12


@pytest.fixture(scope="module")
def tg():
    import pytreegrav_gb300 as tg

    return tg


def rel_rms(a, ref):
    a, ref = np.asarray(a).reshape(len(a), -1), np.asarray(ref).reshape(len(ref), -1)
    return np.sqrt(np.mean(np.sum((a - ref) ** 2, 1))) / np.sqrt(np.mean(np.sum(ref**2, 1)))


def rel_max(a, ref):
    """Worst per-target error, relative to that target's own field (floored at the RMS field, so
    targets whose field cancels to ~0 are judged against the typical magnitude)."""
    a, ref = np.asarray(a).reshape(len(a), -1), np.asarray(ref).reshape(len(ref), -1)
    scale = np.sqrt(np.mean(np.sum(ref**2, 1)))
    mag = np.maximum(np.sqrt(np.sum(ref**2, 1)), scale)
    return np.max(np.sqrt(np.sum((a - ref) ** 2, 1)) / mag)


def plummer(n, rng):
    u = rng.random(n)
    r = 1 / np.sqrt(u ** (-2 / 3) - 1)
    d = rng.normal(size=(n, 3))
    return d / np.linalg.norm(d, axis=1)[:, None] * r[:, None]


@pytest.mark.parametrize("gs", [1, 8, 32])
@pytest.mark.parametrize("quad", [False, True])
@pytest.mark.parametrize("theta", [0.4, 0.7])
def test_walk_vs_golden(tg, golden_walk, gs, quad, theta):
    g = golden_walk
    t = tg.ConstructTree(g["src/pos"], g["src/m"], g["src/h"], quadrupole=True)
    idx = t.TreewalkIndices
    xs, hs = g["src/pos"][idx][:256], g["src/h"][idx][:256]
    for prec, rms_tol, max_tol in (("fp64", FP64_TOL, FP64_TOL), ("fp32", FP32_RMS, FP32_MAX)):
        res = t.fields(xs, hs, True, True, True, quadrupole=quad, group_size=gs, theta=theta, order="given",
                       precision=prec)
        for k in ("potential", "accel", "tidal"):
            ref = g[f"g{gs}_q{int(quad)}_t{theta}/{k}"]
            assert rel_rms(res[k], ref) < rms_tol, (prec, k, rel_rms(res[k], ref))
            assert rel_max(res[k], ref) < max_tol, (prec, k, rel_max(res[k], ref))


def test_frontend_vs_golden(tg, golden_walk):
    g = golden_walk
    x, m, h = g["frontend/pos"], g["frontend/m"], g["frontend/h"]
    for prec, tol in (("fp64", FP64_TOL), ("fp32", FP32_RMS)):
        a = tg.Accel(x, m, h, method="tree", theta=0.7, precision=prec)
        assert rel_rms(a, g["frontend/Accel"]) < tol
        p = tg.Potential(x, m, h, method="tree", theta=0.7, quadrupole=True, precision=prec)
        assert rel_rms(p, g["frontend/Potential"]) < tol
        xt, ht = g["frontend/targets"], g["frontend/h_t"]
        at = tg.AccelTarget(xt, x, m, ht, h, method="tree", theta=0.6, precision=prec)
        assert rel_rms(at, g["frontend/AccelTarget"]) < tol
        tt = tg.TidalTensorTarget(xt, x, m, ht, h, method="tree", theta=0.6, quadrupole=True, precision=prec)
        assert rel_rms(tt, g["frontend/TidalTensorTarget"]) < tol


@pytest.mark.parametrize("quad", [False, True])
@pytest.mark.parametrize("gs", [8, 32])
def test_plummer_1e5_vs_oracle(tg, quad, gs):
    """Self-gravity at 1e5 (Plummer, softened): every target against the oracle's FP64 grouped walk."""
    rng = np.random.default_rng(11)
    n = 100_000
    x = plummer(n, rng)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.005)
    ref, _ = O.self_fields(x, m, h, potential=True, accel=True, theta=0.7, quadrupole=quad, group_size=gs,
                           nthreads=O.num_threads())
    for prec, tol, mtol in (("fp32", FP32_RMS, FP32_MAX), ("fp64", FP64_TOL, FP64_TOL)):
        f = tg.Field(x, m, h, theta=0.7, quadrupole=quad, group_size=gs, precision=prec)
        res = f.evaluate(potential=True, accel=True)
        for k in ("potential", "accel"):
            assert rel_rms(res[k], ref[k]) < tol, (prec, k, rel_rms(res[k], ref[k]))
            assert rel_max(res[k], ref[k]) < mtol, (prec, k, rel_max(res[k], ref[k]))


def test_external_targets_vs_oracle(tg):
    rng = np.random.default_rng(5)
    xs = plummer(50_000, rng)
    ms = rng.random(50_000) / 50_000
    hs = np.exp(rng.normal(np.log(0.003), 0.7, 50_000))
    xt = rng.normal(size=(20_000, 3)) * 2
    ht = np.zeros(20_000)
    ref, _ = O.target_fields(xt, ht, xs, ms, hs, potential=True, accel=True, tidal=True, theta=0.5,
                             quadrupole=True, nthreads=O.num_threads())
    res = tg.Field(xs, ms, hs, theta=0.5, quadrupole=True).evaluate(True, True, True, pos_target=xt,
                                                                    softening_target=ht)
    for k in ref:
        assert rel_rms(res[k], ref[k]) < FP32_RMS, k
        assert rel_max(res[k], ref[k]) < FP32_MAX, k


def test_bruteforce_fp64_bit_exact(tg, golden_bruteforce):
    g = golden_bruteforce
    xs, ms, hs, xt, ht = g["src/pos"], g["src/m"], g["src/h"], g["tgt/pos"], g["tgt/h"]
    r = tg.bruteforce(xt, ht, xs, ms, hs, True, True, True, precision="fp64")
    assert np.array_equal(r["potential"], g["PotentialTarget"])
    assert np.array_equal(r["accel"], g["AccelTarget"])
    assert np.array_equal(r["tidal"], g["TidalTensorTarget"])
    r = tg.bruteforce(None, None, xs, ms, hs, True, True, True, mutual=True, precision="fp64")
    assert np.array_equal(r["potential"], g["Potential_mutual"])
    assert np.array_equal(r["accel"], g["Accel_mutual"])
    assert np.array_equal(r["tidal"], g["TidalTensor_mutual"])


@pytest.mark.parametrize("n", [1000, 4097, 20000])
@pytest.mark.parametrize("soft", ["zero", "uniform", "varying"])
def test_bruteforce_fp32(tg, n, soft):
    """FP32 direct sum within the sqrt(N) accumulation bound the reference uses (1e-5*sqrt(N/1000))."""
    rng = np.random.default_rng(42)
    x = rng.normal(size=(n, 3))
    m = np.ones(n) / n
    h = {"zero": np.zeros(n), "uniform": np.full(n, 0.05), "varying": 2.0 * n ** (-1 / 3) * rng.random(n)}[soft]
    ref = O.bruteforce(x, h, x, m, h, True, True, False, mutual=True, nthreads=O.num_threads())
    got = tg.bruteforce(None, None, x, m, h, True, True, False, mutual=True, precision="fp32")
    tol = 1e-5 * np.sqrt(n / 1000)
    assert np.abs(got["potential"] - ref["potential"]).max() / np.abs(ref["potential"]).max() < tol
    e = np.sqrt(np.sum((got["accel"] - ref["accel"]) ** 2, 1)) / np.sqrt(np.sum(ref["accel"] ** 2, 1))
    assert e.max() < tol


def test_tree_vs_bruteforce_accuracy(tg):
    """The reference's integration bar (tree_test.py): RMS force and potential error < 0.02."""
    rng = np.random.default_rng(42)
    n = 40_000
    x = rng.random((n, 3))
    m = np.ones(n) / n
    h = np.full(n, 0.01)
    a_t = tg.Accel(x, m, h, method="tree")
    a_b = tg.Accel(x, m, h, method="bruteforce")
    p_t = tg.Potential(x, m, h, method="tree")
    p_b = tg.Potential(x, m, h, method="bruteforce")
    assert np.sqrt(np.mean(np.sum((a_t - a_b) ** 2, 1))) < 0.02
    assert np.std(p_t - p_b) < 0.02


@pytest.mark.parametrize("quad", [False, True])
@pytest.mark.parametrize("G", [16, 32])
def test_tree_grouping_vs_oracle(tg, quad, G):
    """The engine's tree grouping: the oracle walks the same groups (grouping rule restated in
    oracle.tree_groups), so FP64 agrees to rounding and FP32 to the FP32 bar."""
    rng = np.random.default_rng(23)
    n = 60_000
    u = rng.random(n)
    r = 1 / np.sqrt(u ** (-2 / 3) - 1)
    keep = r < 50
    x = plummer(n, np.random.default_rng(23))[keep]
    n = len(x)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.005)
    ot = O.OracleTree(x, m, h, quadrupole=True)
    S, C = O.tree_groups(ot, G)
    idx = ot.TreewalkIndices
    ref_sorted = O.fields_groups(ot, ot.Coordinates[:n], ot.Softenings[:n], S, C, True, True, True, quad, 0.7,
                                 nthreads=O.num_threads())
    t = tg.ConstructTree(x, m, h, quadrupole=True)
    for prec, tol, mtol in (("fp64", FP64_TOL, FP64_TOL), ("fp32", FP32_RMS, FP32_MAX)):
        res = t.fields(potential=True, accel=True, tidal=True, quadrupole=quad, group_size=G, theta=0.7,
                       grouping="tree", precision=prec)
        for k in res:
            ref = np.empty_like(ref_sorted[k])
            ref[idx] = ref_sorted[k]
            assert rel_rms(res[k], ref) < tol, (prec, k, rel_rms(res[k], ref))
            assert rel_max(res[k], ref) < mtol, (prec, k, rel_max(res[k], ref))
    st = t.last_walk_stats()
    assert st[3] == len(S), "GPU and restated grouping differ in group count"


@pytest.mark.parametrize("quad", [False, True])
@pytest.mark.parametrize("gs", [8, 32])
@pytest.mark.parametrize("grouping", ["blocks", "tree"])
def test_tidal_alone_fp32_vs_oracle(tg, quad, gs, grouping):
    """The tidal tensor requested alone takes its own FP32 walk (paired sweeps over leaves and
    quadrupole nodes): against the oracle's FP64 grouped walk, and against the tidal part of the
    all-fields walk, at the FP32 tolerances."""
    rng = np.random.default_rng(31)
    n = 60_000
    x = plummer(n, rng)
    keep = np.linalg.norm(x, axis=1) < 50
    x = x[keep]
    n = len(x)
    m = rng.random(n) / n
    h = np.full(n, 0.005)
    ot = O.OracleTree(x, m, h, quadrupole=True)
    idx = ot.TreewalkIndices
    if grouping == "tree":
        S, C = O.tree_groups(ot, gs)
    else:
        S = np.arange(0, n, gs, dtype=np.int64)
        C = np.minimum(gs, n - S)
    ref_sorted = O.fields_groups(ot, ot.Coordinates[:n], ot.Softenings[:n], S, C, False, False, True, quad, 0.7,
                                 nthreads=O.num_threads())["tidal"]
    ref = np.empty_like(ref_sorted)
    ref[idx] = ref_sorted
    t = tg.ConstructTree(x, m, h, quadrupole=True)
    alone = t.fields(tidal=True, quadrupole=quad, group_size=gs, theta=0.7, grouping=grouping)["tidal"]
    every = t.fields(potential=True, accel=True, tidal=True, quadrupole=quad, group_size=gs, theta=0.7,
                     grouping=grouping)["tidal"]
    assert rel_rms(alone, ref) < FP32_RMS and rel_max(alone, ref) < FP32_MAX
    assert rel_rms(alone, every) < FP32_RMS
    assert np.allclose(alone, np.swapaxes(alone, 1, 2))  # symmetric
