"""Bounded device loops made to run out, a corrupted tree caught by the walk arena's check, the
split walk of heavy groups, and FP32 brute force at the softening boundary.

Every bounded wait or loop of the library has a runtime override (tg_set_loop_limits, measurement
header). Each test below sets one to a tiny value, checks the status the call returns, restores the
built-in bounds, and checks that the next call on the same library gives the right answer. None of
these cases faults or hangs the GPU: a look-back that gives up leaves the identity permutation (every
later index stays in range), a walk or column walk that runs out stops with its group's rows
unwritten and a status bit set, and the corrupted tree keeps every link inside the arena.
"""

import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import pytreegrav_gb300 as tg
    from pytreegrav_gb300 import _lib

    L = _lib.load()
    L.tg_set_loop_limits.argtypes = [ctypes.c_int64] * 4
    L.tg_set_loop_limits.restype = ctypes.c_int
    yield tg, _lib, L
    L.tg_set_loop_limits(0, 0, 0, 0)


def plummer(n, seed):
    from pytreegrav_gb300 import synthetic

    return synthetic.plummer(n, seed)


def rel_rms(a, ref):
    a, ref = np.asarray(a).reshape(len(a), -1), np.asarray(ref).reshape(len(ref), -1)
    return np.sqrt(np.mean(np.sum((a - ref) ** 2, 1))) / np.sqrt(np.mean(np.sum(ref**2, 1)))


def build(_lib, L, x, m, h, quad=True):
    t = ctypes.c_void_p()
    rc = L.tg_tree_build(_lib.ptr(x), _lib.ptr(m), _lib.ptr(h), len(x), int(quad), 1, _lib.TG_MEM_HOST, None,
                         ctypes.byref(t))
    return rc, t


def test_sort_lookback_runs_out(env):
    """One poll per look-back word: a build either completes (then its tree is the oracle's) or
    returns TG_ERR_QUEUE_TIMEOUT; over several tries on 1e6 keys (489 concurrent tiles per pass) at
    least one runs out. tg_morton_order the same. Then the default bound builds the right tree."""
    tg, _lib, L = env
    n = 1_000_000
    x = plummer(n, 41)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.005)
    ref = O.OracleTree(x, m, h, quadrupole=True)
    timeouts = 0
    L.tg_set_loop_limits(1, 0, 0, 0)
    try:
        for _ in range(4):
            rc, t = build(_lib, L, x, m, h)
            if rc == _lib.TG_OK:
                tree = tg.Octree._from_handle(t, True)
                assert np.array_equal(tree.TreewalkIndices, ref.TreewalkIndices)
                del tree
            else:
                assert rc == _lib.TG_ERR_QUEUE_TIMEOUT, rc
                timeouts += 1
            perm = np.empty(n, np.int64)
            rc = L.tg_morton_order(_lib.ptr(x), n, _lib.TG_MEM_HOST, _lib.ptr(perm), None)
            if rc == _lib.TG_OK:
                assert np.array_equal(perm, O.morton_order(x))
            else:
                assert rc == _lib.TG_ERR_QUEUE_TIMEOUT, rc
                timeouts += 1
    finally:
        L.tg_set_loop_limits(0, 0, 0, 0)
    assert timeouts > 0
    tree = tg.ConstructTree(x, m, h, quadrupole=True)
    assert np.array_equal(tree.TreewalkIndices, ref.TreewalkIndices)
    assert np.array_equal(tree.Masses, ref.Masses)


def test_walk_step_limit_runs_out(env):
    tg, _lib, L = env
    n = 20_000
    x = plummer(n, 42)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.01)
    tree = tg.ConstructTree(x, m, h, quadrupole=True)
    out = np.empty((n, 3))
    L.tg_set_loop_limits(0, 1, 0, 0)
    try:
        for grouping in (_lib.TG_GROUP_BLOCKS, _lib.TG_GROUP_TREE):
            rc = L.tg_tree_fields(tree._h, None, None, n, _lib.TG_FIELD_ACCEL, 1, 0.7, 1.0, 8, grouping,
                                  _lib.TG_ORDER_TREE, _lib.TG_FP32, None, _lib.TG_MEM_HOST, _lib.ptr(out), None)
            assert rc == _lib.TG_ERR_ITER_LIMIT, rc
    finally:
        L.tg_set_loop_limits(0, 0, 0, 0)
    ref, _ = O.self_fields(x, m, h, accel=True, theta=0.7, quadrupole=True, nthreads=O.num_threads())
    a = tree.fields(accel=True, quadrupole=True, theta=0.7)["accel"]
    assert rel_rms(a, ref["accel"]) < 1e-5


def test_column_visit_limit_runs_out(env):
    tg, _lib, L = env
    n = 5_000
    x = plummer(n, 43)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.02)
    tree = tg.ConstructTree(x, m, h)
    rays = np.vstack([np.eye(3), -np.eye(3)])
    L.tg_set_loop_limits(0, 0, 1, 0)
    try:
        with pytest.raises(_lib.GravityError):
            tree.column_density(x[:100], rays)
    finally:
        L.tg_set_loop_limits(0, 0, 0, 0)
    idx = tree.TreewalkIndices
    ot = O.OracleTree(x, m, h)
    assert np.array_equal(tree.column_density(x[idx][:100], rays), O.column_rays(ot, x[idx][:100], rays))


@pytest.mark.parametrize("quad", [False, True])
def test_heavy_group_split_walk(env, quad):
    """With a split budget of 8 list entries nearly every group of 8 goes through the split walk
    (top walk, items on all warps, reduction in item order): the accepted set is pytreegrav's, so FP64
    agrees with the oracle to rounding and FP32 to the walk bar; two runs are bit-identical; the
    unsplit walk agrees to FP32 rounding."""
    tg, _lib, L = env
    n = 50_000
    x = plummer(n, 44)
    m = np.random.default_rng(45).random(n) / n
    h = np.full(n, 0.005)
    ref, _ = O.self_fields(x, m, h, potential=True, accel=True, tidal=True, theta=0.7, quadrupole=quad,
                           nthreads=O.num_threads())
    tree = tg.ConstructTree(x, m, h, quadrupole=True)
    kw = dict(potential=True, accel=True, tidal=True, quadrupole=quad, group_size=8, theta=0.7)
    whole = tree.fields(**kw)
    L.tg_set_loop_limits(0, 0, 0, 8)
    try:
        split = [tree.fields(precision="fp32", **kw) for _ in range(2)]
        split64 = tree.fields(precision="fp64", **kw)
    finally:
        L.tg_set_loop_limits(0, 0, 0, 0)
    for k in ("potential", "accel", "tidal"):
        assert np.array_equal(split[0][k], split[1][k]), k
        assert rel_rms(split[0][k], ref[k]) < 1e-5, k
        assert rel_rms(split64[k], ref[k]) < 1e-12, k
        assert rel_rms(split[0][k], whole[k]) < 1e-6, k


def test_heavy_groups_of_blocks_at_1e6(env):
    """The default grouping at 1e6 Plummer particles (its few heavy groups split at the built-in
    budget): against the oracle walking the heaviest groups, whose targets straddle a jump of the
    Morton curve."""
    tg, _lib, L = env
    n = 1_000_000
    x = plummer(n, 20261203)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.005)
    ot = O.OracleTree(x, m, h, quadrupole=True)
    idx = ot.TreewalkIndices
    ni, _ = ot.walk_counts(x[idx], h[idx], group_size=8, theta=0.7, nthreads=O.num_threads())
    heavy = np.argsort(ni)[::-1][:8]  # the 8 heaviest groups of 8
    starts = heavy.astype(np.int64) * 8
    counts = np.minimum(8, n - starts)
    ref = O.fields_groups(ot, x[idx], h[idx], starts, counts, True, True, False, True, 0.7, nthreads=O.num_threads())
    tree = tg.ConstructTree(x, m, h, quadrupole=True)
    got = tree.fields(potential=True, accel=True, quadrupole=True, group_size=8, theta=0.7)
    rows = np.concatenate([np.arange(s, s + c) for s, c in zip(starts, counts)])
    for k in ("potential", "accel"):
        assert rel_rms(got[k][idx[rows]], ref[k][rows]) < 1e-5, k


def test_corrupted_links_caught_by_the_arena_check(env):
    """A tree whose links are rewired inside the arena (a particle's NextBranch pointed at itself, a
    loop) no longer forms a valid octree: the walk arena's device check reports it as an error
    instead of walking it, and the library keeps working."""
    torch = pytest.importorskip("torch")
    tg, _lib, L = env
    n = 5_000
    x = plummer(n, 46)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.01)
    tree = tg.ConstructTree(x, m, h, quadrupole=True)
    first, nxt = tree.FirstSubnode, tree.NextBranch
    N, hi = tree.NumParticles, tree.node_hi
    # a node whose first child is a particle: that particle's link made a loop
    j = next(f for f in range(N, hi) if 0 <= first[f] < N)
    info = _lib.TreeInfo()
    _lib.check(L.tg_tree_info_get(tree._h, ctypes.byref(info)))

    class View:  # the tree's NextBranch array on the device, as a torch tensor (no copy)
        __cuda_array_interface__ = {"shape": (hi,), "typestr": "<i8", "data": (info.next, False), "version": 2}

    dev_next = torch.as_tensor(View(), device="cuda")
    dev_next[int(first[j])] = int(first[j])
    torch.cuda.synchronize()
    with pytest.raises(_lib.GravityError, match="valid octree"):
        tree.fields(accel=True, quadrupole=True, theta=0.7)  # pytreegrav's grouping: no chain is followed first
    del dev_next
    a = tg.Accel(x, m, h, quadrupole=True, method="tree")
    ref, _ = O.self_fields(x, m, h, accel=True, theta=0.7, quadrupole=True, nthreads=O.num_threads())
    assert rel_rms(a, ref["accel"]) < 1e-5


@pytest.mark.parametrize("nt", [1, 3, 1001])
def test_bruteforce_fp32_at_the_softening_boundary(env, nt):
    """FP32 brute force with targets at r = max(h_i, h_j) * (1 +- 1e-5) from sources, where the paired
    point-mass path and the softened path meet, and an odd target count, against the oracle at the
    reference's sqrt(N) bound."""
    tg, _lib, L = env
    rng = np.random.default_rng(47)
    ns = 2000
    xs = rng.normal(size=(ns, 3))
    hs = 0.05 + 0.05 * rng.random(ns)
    ms = rng.random(ns) / ns
    src = rng.integers(0, ns, nt)
    d = rng.normal(size=(nt, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    ht = 0.05 + 0.05 * rng.random(nt)
    r = np.maximum(hs[src], ht) * (1 + 1e-5 * rng.choice([-1.0, 1.0], nt))
    xt = xs[src] + d * r[:, None]
    ref = O.bruteforce(xt, ht, xs, ms, hs, True, True, False, nthreads=O.num_threads())
    got = tg.bruteforce(xt, ht, xs, ms, hs, True, True, False, precision="fp32")
    tol = 1e-5 * np.sqrt(ns / 1000)
    assert np.abs(got["potential"] - ref["potential"]).max() / np.abs(ref["potential"]).max() < tol
    e = np.sqrt(np.sum((got["accel"] - ref["accel"]) ** 2, 1)) / np.sqrt(np.sum(ref["accel"] ** 2, 1))
    assert e.max() < tol
