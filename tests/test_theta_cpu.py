"""Learned opening angle, host side: the numpy checker's gradients against finite differences, the
training tables' interpolation, model files and the feature normalisation."""

import numpy as np
import pytest

import mlp_ref as R
from pytreegrav_gb300 import _lib, theta


def test_layout_matches_library():
    assert R.NP == _lib.TG_MLP_NPARAM == theta.NP


def test_reference_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = theta.ThetaModel.init_params(1).astype(np.float64) + rng.normal(0, 0.05, R.NP)
    x = rng.normal(size=(7, R.NF))
    dy = rng.normal(size=7)
    g = R.backward(p, x, dy)
    f = lambda q: float(np.dot(dy, R.forward(q, x)[0]))
    for i in rng.choice(R.NP, 60, replace=False):
        e = np.zeros(R.NP)
        e[i] = 1e-6
        num = (f(p + e) - f(p - e)) / 2e-6
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(num), i


def test_reference_loss_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    n, K = 9, len(theta.GRID)
    lc = np.cumsum(-rng.random((n, K)), axis=1)  # cost falls with theta
    le = np.cumsum(rng.random((n, K)) * 2, axis=1) - 8  # error grows with theta
    lam = 10 ** rng.uniform(-1, 2, n)
    y = rng.normal(size=n)
    t0, dt = float(theta.GRID[0]), float(theta.GRID[1] - theta.GRID[0])
    _, dy = R.theta_loss(y, lc, le, lam, t0, dt, theta.THETA_MIN, theta.THETA_MAX)
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1e-7
        num = (R.theta_loss(y + e, lc, le, lam, t0, dt, theta.THETA_MIN, theta.THETA_MAX)[0] -
               R.theta_loss(y - e, lc, le, lam, t0, dt, theta.THETA_MIN, theta.THETA_MAX)[0]) / 2e-7
        assert abs(num - dy[i]) <= 1e-7 + 1e-4 * abs(num)


def test_table_interpolation_hits_grid_points():
    rng = np.random.default_rng(2)
    tab = rng.normal(size=(5, len(theta.GRID)))
    for k, th in enumerate(theta.GRID):
        np.testing.assert_allclose(theta.table_at(tab, np.full(5, th)), np.exp(tab[:, k]), rtol=1e-12)


def test_model_file_round_trip(tmp_path):
    m = theta.ThetaModel(theta.ThetaModel.init_params(3), np.arange(16), np.ones(16), 0.25, {"a": 1})
    m.save(tmp_path / "m.npz")
    m2 = theta.ThetaModel.load(tmp_path / "m.npz")
    assert np.array_equal(m.params, m2.params) and m2.log10_lambda == 0.25 and m2.meta == {"a": 1}


def test_feature_stats_fix_the_lambda_slot_and_constant_features():
    d = dict(features=np.column_stack([np.random.default_rng(4).normal(size=(50, 15)), np.ones(50)]))
    d["features"][:, _lib.TG_THETA_FEAT_LAMBDA] = 0
    mean, std = theta.feature_stats([d])
    lo, hi = theta.LOG10_LAMBDA_RANGE
    assert mean[_lib.TG_THETA_FEAT_LAMBDA] == pytest.approx(0.5 * (lo + hi))
    assert std[15] == 1.0 and np.all(std > 0)


def test_shipped_model_loads_if_present():
    import os

    if not os.path.exists(theta.DEFAULT_MODEL):
        pytest.skip("no trained model in the package yet")
    m = theta.ThetaModel.load()
    assert m.params.shape == (R.NP,) and np.all(np.isfinite(m.params))
    assert theta.LOG10_LAMBDA_RANGE[0] <= m.log10_lambda <= theta.LOG10_LAMBDA_RANGE[1]
