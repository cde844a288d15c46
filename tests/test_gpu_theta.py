"""Learned opening angle on the GPU: the training kernels against the numpy checker, BF16 inference
against the FP32 forward pass, features and per-group counters, and the learned walk."""

import ctypes
import os

import numpy as np
import pytest

import mlp_ref as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from pytreegrav_gb300 import _lib, theta

    return torch, _lib, _lib.load(), theta


def vp(t):
    return ctypes.c_void_p(t.data_ptr())


def dev(torch, a, dtype=None):
    a = np.ascontiguousarray(a, dtype or np.float32)
    return torch.from_numpy(a).cuda()


def test_forward_and_backward_match_numpy(env):
    torch, _lib, L, theta = env
    rng = np.random.default_rng(0)
    n = 333
    p = (theta.ThetaModel.init_params(5) + rng.normal(0, 0.02, R.NP)).astype(np.float32)
    x = rng.normal(size=(n, R.NF)).astype(np.float32)
    dy = rng.normal(size=n).astype(np.float32)
    P, X, DY = dev(torch, p), dev(torch, x), dev(torch, dy)
    y = torch.empty(n, dtype=torch.float32, device="cuda")
    acts = torch.empty((n, 128), dtype=torch.float32, device="cuda")
    work = torch.empty((n, 128), dtype=torch.float32, device="cuda")
    grad = torch.empty(R.NP, dtype=torch.float32, device="cuda")
    assert L.tg_mlp_forward(vp(P), vp(X), n, vp(acts), vp(y), None) == 0
    assert L.tg_mlp_backward(vp(P), vp(X), vp(acts), vp(DY), n, vp(work), vp(grad), None) == 0
    torch.cuda.synchronize()
    y_ref, z1, z2 = R.forward(p.astype(np.float64), x.astype(np.float64))
    np.testing.assert_allclose(y.cpu().numpy(), y_ref, rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(acts.cpu().numpy()[:, :64], z1, rtol=1e-4, atol=1e-4)
    g_ref = R.backward(p.astype(np.float64), x.astype(np.float64), dy.astype(np.float64))
    g = grad.cpu().numpy()
    scale = np.abs(g_ref).max()
    assert np.abs(g - g_ref).max() <= 1e-4 * scale, np.abs(g - g_ref).max() / scale


def test_loss_and_adam_match_numpy(env):
    torch, _lib, L, theta = env
    rng = np.random.default_rng(1)
    n, K = 1000, len(theta.GRID)
    lc = np.cumsum(-rng.random((n, K)), axis=1).astype(np.float32)
    le = (np.cumsum(rng.random((n, K)) * 2, axis=1) - 8).astype(np.float32)
    lam = (10 ** rng.uniform(-1, 2, n)).astype(np.float32)
    y = rng.normal(size=n).astype(np.float32)
    Y, LC, LE, LAM = (dev(torch, a) for a in (y, lc, le, lam))
    dy = torch.empty(n, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    t0, dt = float(theta.GRID[0]), float(theta.GRID[1] - theta.GRID[0])
    assert L.tg_theta_loss(vp(Y), vp(LC), vp(LE), vp(LAM), n, K, t0, dt, theta.THETA_MIN, theta.THETA_MAX, vp(dy),
                           vp(loss), None) == 0
    torch.cuda.synchronize()
    l_ref, dy_ref = R.theta_loss(y.astype(np.float64), lc.astype(np.float64), le.astype(np.float64),
                                 lam.astype(np.float64), t0, dt, theta.THETA_MIN, theta.THETA_MAX)
    assert float(loss.item()) == pytest.approx(l_ref, rel=1e-4)
    np.testing.assert_allclose(dy.cpu().numpy(), dy_ref, rtol=1e-3, atol=1e-7 * np.abs(dy_ref).max())
    p = rng.normal(size=R.NP).astype(np.float32)
    g = rng.normal(size=R.NP).astype(np.float32)
    m = rng.normal(size=R.NP).astype(np.float32) * 0.1
    v = rng.random(R.NP).astype(np.float32) * 0.1
    P, G_, M, V = (dev(torch, a) for a in (p, g, m, v))
    assert L.tg_adam_step(vp(P), vp(G_), vp(M), vp(V), R.NP, 1e-3, 0.9, 0.999, 1e-8, 7, None) == 0
    torch.cuda.synchronize()
    p_ref, m_ref, v_ref = R.adam(p.astype(np.float64), g, m, v, 1e-3, 0.9, 0.999, 1e-8, 7)
    np.testing.assert_allclose(P.cpu().numpy(), p_ref, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(M.cpu().numpy(), m_ref, rtol=1e-5, atol=1e-7)


def test_bf16_inference_matches_fp32_forward(env):
    torch, _lib, L, theta = env
    rng = np.random.default_rng(2)
    n = 1000 + 7  # not a multiple of the 16-row tile
    p = (theta.ThetaModel.init_params(9) + rng.normal(0, 0.02, R.NP)).astype(np.float32)
    mean = rng.normal(size=R.NF).astype(np.float32)
    std = (0.5 + rng.random(R.NF)).astype(np.float32)
    feat = (mean + std * rng.normal(size=(n, R.NF))).astype(np.float32)
    model = theta.ThetaModel(p, mean, std)
    l10 = 0.4
    th = theta.predict(model, feat, l10)
    xn = (feat.astype(np.float64) - mean) / std
    xn[:, _lib.TG_THETA_FEAT_LAMBDA] = (l10 - mean[_lib.TG_THETA_FEAT_LAMBDA]) / std[_lib.TG_THETA_FEAT_LAMBDA]
    y, _, _ = R.forward(p.astype(np.float64), xn)
    th_ref = theta.THETA_MIN + (theta.THETA_MAX - theta.THETA_MIN) * R.sigmoid(y)
    err = np.abs(th - th_ref)
    assert err.max() < 0.02 and err.mean() < 0.004, (err.max(), err.mean())
    model.close()


@pytest.fixture(scope="module")
def plummer_tree(env):
    torch, _lib, L, theta = env
    from pytreegrav_gb300 import synthetic

    n = 200_000
    x = synthetic.plummer(n, 7)
    tree, keep = theta._tree_device(torch, x, np.full(n, 1.0 / n), np.full(n, 0.005), True)
    yield tree, keep, x
    L.tg_tree_free(tree)


def test_features_and_group_counters(env, plummer_tree):
    torch, _lib, L, theta = env
    tree, keep, x = plummer_tree
    n = len(x)
    first, count, node = theta.groups_of(tree, 32)
    assert count.sum() == n and np.all(count >= 1) and np.all(count <= 32)
    assert np.all(np.diff(first) > 0) and first[0] == 0
    f = theta.features(tree, 32, True)
    assert f.shape == (len(first), R.NF) and np.all(np.isfinite(f))
    assert np.allclose(f[:, 0], np.log2(count))
    assert np.all(f[:, _lib.TG_THETA_FEAT_LAMBDA] == 0) and np.all(f[:, 14] == 1)
    out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    assert L.tg_tree_record_group_stats(tree, 1) == 0
    assert L.tg_tree_fields(tree, None, None, n, _lib.TG_FIELD_ACCEL, 1, 0.7, 1.0, 32, _lib.TG_GROUP_TREE,
                            _lib.TG_ORDER_TREE, _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, vp(out), None) == 0
    stats = np.empty((len(first), 3), np.uint32)
    assert L.tg_tree_last_group_stats(tree, _lib.ptr(stats), _lib.TG_MEM_HOST, None) == 0
    assert L.tg_tree_record_group_stats(tree, 0) == 0
    v = [ctypes.c_int64() for _ in range(4)]
    L.tg_tree_last_walk_stats(tree, *[ctypes.byref(q) for q in v])
    # the walk counts an interaction per (entry, target of the group)
    total = int(((stats[:, 0].astype(np.int64) + stats[:, 1]) * count).sum())
    assert total == v[0].value
    assert int(stats[:, 2].astype(np.int64).sum()) >= len(first)


def test_learned_walk_without_model_is_the_plain_walk(env, plummer_tree):
    torch, _lib, L, theta = env
    tree, keep, x = plummer_tree
    n = len(x)
    a = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    b = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    assert L.tg_tree_fields(tree, None, None, n, _lib.TG_FIELD_ACCEL, 1, 0.7, 1.0, 32, _lib.TG_GROUP_TREE,
                            _lib.TG_ORDER_TREE, _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, vp(a), None) == 0
    assert L.tg_tree_fields_learned(tree, _lib.TG_FIELD_ACCEL, 1, 1.0, 32, None, 0.0, 0.7, _lib.TG_MEM_DEVICE, vp(b),
                                    None) == 0
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_groups_over_the_error_budget_are_rewalked_at_the_global_theta(env, plummer_tree):
    """A budget below every group's estimate sends every group back through the walk at the
    global theta: the result is then the plain walk's, bit for bit. Budget 0 (off) leaves the
    learned result alone; the per-group estimates are finite and non-negative."""
    torch, _lib, L, theta = env
    tree, keep, x = plummer_tree
    n = len(x)
    model = theta.ThetaModel.load()
    l10 = theta.default_lambda(model, True)
    plain = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    learned = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    rewalked = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    assert L.tg_tree_fields(tree, None, None, n, _lib.TG_FIELD_ACCEL, 1, 0.7, 1.0, 32, _lib.TG_GROUP_TREE,
                            _lib.TG_ORDER_TREE, _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, vp(plain), None) == 0
    h = model.handle()
    try:
        assert L.tg_theta_model_set_error_budget(h, 0.0) == 0
        assert L.tg_tree_record_group_stats(tree, 1) == 0
        assert L.tg_tree_fields_learned(tree, _lib.TG_FIELD_ACCEL, 1, 1.0, 32, h, l10, 0.7, _lib.TG_MEM_DEVICE,
                                        vp(learned), None) == 0
        first, _, _ = theta.groups_of(tree, 32)
        eta = np.empty(len(first), np.float32)
        assert L.tg_tree_last_group_error(tree, _lib.ptr(eta), _lib.TG_MEM_HOST, None) == 0
        assert L.tg_tree_record_group_stats(tree, 0) == 0
        assert np.all(np.isfinite(eta)) and np.all(eta >= 0) and eta.max() > 0
        assert L.tg_theta_model_set_error_budget(h, float(eta[eta > 0].min()) * 1e-3) == 0
        assert L.tg_tree_fields_learned(tree, _lib.TG_FIELD_ACCEL, 1, 1.0, 32, h, l10, 0.7, _lib.TG_MEM_DEVICE,
                                        vp(rewalked), None) == 0
        torch.cuda.synchronize()
        assert torch.equal(rewalked, plain)
        assert not torch.equal(learned, plain)
    finally:
        model.close()


def test_learned_walk_is_its_parts_and_repeats(env, plummer_tree):
    """tg_tree_fields_learned with the shipped tolerance model (no error budget) equals its parts run
    one by one, bit for bit: the features (tg_theta_features), the network (tg_theta_infer), the
    tolerances (tg_theta_tolerances), then tg_tree_fields_grouped at the model's angle cap with those
    tolerances -- inside the learned call the inference kernel writes the tolerances itself. The
    features (whose top-level frontier is listed in node order) and the learned walk repeat bit for
    bit."""
    torch, _lib, L, theta = env
    tree, keep, x = plummer_tree
    n = len(x)
    model = theta.ThetaModel.load()
    if model.kind != "tolerance":
        pytest.skip("the shipped model is not a tolerance model")
    l10 = theta.default_lambda(model, True)
    f1 = theta.features(tree, 32, True)
    f2 = theta.features(tree, 32, True)
    assert np.array_equal(f1, f2)
    u = torch.from_numpy(theta.predict(model, f1, l10)).cuda()
    tol = torch.empty(len(f1), dtype=torch.float32, device="cuda")
    assert L.tg_theta_tolerances(tree, 32, 1, vp(u), vp(tol), None) == 0
    parts = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    assert L.tg_tree_fields_grouped(tree, _lib.TG_FIELD_ACCEL, 1, 1.0, 32, model.theta_max, None, vp(tol),
                                    _lib.TG_MEM_DEVICE, vp(parts), None) == 0
    a = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    b = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    h = model.handle()
    try:
        assert L.tg_theta_model_set_error_budget(h, 0.0) == 0
        for out in (a, b):
            assert L.tg_tree_fields_learned(tree, _lib.TG_FIELD_ACCEL, 1, 1.0, 32, h, l10, 0.7, _lib.TG_MEM_DEVICE,
                                            vp(out), None) == 0
        torch.cuda.synchronize()
        assert torch.equal(a, b)
        assert torch.equal(a, parts)
    finally:
        model.close()


def test_shipped_model_error_budget_rewalks_few_groups(env, plummer_tree):
    """The shipped budget (twice the worst estimate over the training systems) leaves a held-out
    Plummer system's groups alone, or nearly so."""
    torch, _lib, L, theta = env
    tree, keep, x = plummer_tree
    model = theta.ThetaModel.load()
    if model.error_budget <= 0:
        pytest.skip("the shipped model has no error budget")
    eta = theta.group_errors(model, x, 0.005, True)
    assert np.mean(eta > model.error_budget) < 0.01
    model.close()


@pytest.mark.parametrize("quad", [1, 0])
def test_shipped_model_beats_the_plain_walk_at_equal_error(env, quad):
    """On a Plummer system outside the training set, the learned walk at the model's default
    lambda keeps the plain theta = 0.7 walk's RMS force error (FP64 brute force judge) with at most
    0.6 of its interactions."""
    torch, _lib, L, theta = env
    if not os.path.exists(theta.DEFAULT_MODEL):
        pytest.skip("no trained model in the package")
    from pytreegrav_gb300 import synthetic

    model = theta.ThetaModel.load()
    n = 300_000
    x = synthetic.plummer(n, 11)
    tree, keep = theta._tree_device(torch, x, np.full(n, 1.0 / n), np.full(n, 0.005), quad)
    try:
        idx = np.sort(np.random.default_rng(3).choice(n, 5000, replace=False))
        pt = dev(torch, x[idx], np.float64)
        ht = dev(torch, np.full(len(idx), 0.005), np.float64)
        ref = torch.empty((len(idx), 3), dtype=torch.float64, device="cuda")
        assert L.tg_bruteforce(vp(pt), vp(ht), len(idx), vp(keep[0]), vp(keep[1]), vp(keep[2]), n,
                               _lib.TG_FIELD_ACCEL, 0, 1.0, _lib.TG_FP64, _lib.TG_MEM_DEVICE, vp(ref), None) == 0
        ref = ref.cpu().numpy()
        rms = np.sqrt(np.mean(np.sum(ref ** 2, 1)))
        out = torch.empty((n, 3), dtype=torch.float64, device="cuda")

        def err_and_interactions():
            torch.cuda.synchronize()
            a = out.cpu().numpy()[idx]
            v = [ctypes.c_int64() for _ in range(4)]
            L.tg_tree_last_walk_stats(tree, *[ctypes.byref(q) for q in v])
            return np.sqrt(np.mean(np.sum((a - ref) ** 2, 1))) / rms, v[0].value

        assert L.tg_tree_fields(tree, None, None, n, _lib.TG_FIELD_ACCEL, quad, 0.7, 1.0, 32, _lib.TG_GROUP_TREE,
                                _lib.TG_ORDER_TREE, _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, vp(out), None) == 0
        e_plain, i_plain = err_and_interactions()
        assert L.tg_tree_fields_learned(tree, _lib.TG_FIELD_ACCEL, quad, 1.0, 32, model.handle(),
                                        theta.default_lambda(model, quad), 0.7, _lib.TG_MEM_DEVICE, vp(out),
                                        None) == 0
        e_learned, i_learned = err_and_interactions()
    finally:
        L.tg_tree_free(tree)
        model.close()
    assert e_learned <= e_plain, (e_learned, e_plain)
    # monopole walks gain less (their error falls off one order slower with distance)
    assert i_learned <= (0.6 if quad else 0.75) * i_plain, (i_learned, i_plain)


def test_training_loop_end_to_end(env):
    """theta.collect + theta.train + theta.calibrate on three small systems (a Plummer sphere, a
    clustered mixture and a uniform cube, 2e5 particles each): the loss falls, and the trained model,
    on a held-out Plummer system, stays within 1.25x the plain theta = 0.7 walk's RMS force error
    (FP64 brute force judge) with at most 0.85 of its interactions."""
    torch, _lib, L, theta = env
    import pytreegrav_gb300 as pg
    from pytreegrav_gb300 import synthetic

    k = 200_000
    systems = [("plummer", synthetic.plummer(k, 301), 0.005), ("clustered", synthetic.clustered(k, 302), 0.002),
               ("uniform", synthetic.uniform(k, 304), 0.01)]
    data = [theta.collect(x, np.full(len(x), 1.0 / len(x)), np.full(len(x), soft), quadrupole=True, sample=0.5,
                          seed=i, label=label) for i, (label, x, soft) in enumerate(systems)]
    model = theta.train(data, steps=1500, batch=8192, log_every=100, verbose=False)
    hist = [v for _, v in model.meta["history"]]
    ratios = theta.calibrate(model, data, target_ratio=1.0)
    n = 200_000
    x = synthetic.plummer(n, 303)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.005)
    samp = np.random.default_rng(4).choice(n, 3000, replace=False)
    ref = pg.bruteforce(x[samp], h[samp], x, m, h, accel=True, precision="fp64")["accel"]
    rms = np.sqrt(np.mean(np.sum(ref ** 2, 1)))
    tree = pg.ConstructTree(x, m, h, quadrupole=True)
    plain = tree.fields(accel=True, quadrupole=True, theta=0.7, group_size=32, grouping="tree")["accel"]
    i_plain = tree.last_walk_stats()[0]
    learned = tree.fields(accel=True, quadrupole=True, theta=0.7, learned=model)["accel"]
    i_learned = tree.last_walk_stats()[0]
    e_plain = np.sqrt(np.mean(np.sum((plain[samp] - ref) ** 2, 1))) / rms
    e_learned = np.sqrt(np.mean(np.sum((learned[samp] - ref) ** 2, 1))) / rms
    print(f"\ntraining loop: loss {hist[0]:.3g} -> {hist[-1]:.3g}; log10 lambda {model.log10_lambda:.2f}; predicted "
          f"(error, cost) ratios {[(round(a, 3), round(b, 3)) for a, b in ratios]}; held out: plain {e_plain:.2e} "
          f"({i_plain / n:.0f}/target), learned {e_learned:.2e} ({i_learned / n:.0f}/target)")
    model.close()
    assert hist[-1] < hist[0], hist
    assert e_learned <= 1.25 * e_plain, (e_learned, e_plain)
    assert i_learned <= 0.85 * i_plain, (i_learned, i_plain)
