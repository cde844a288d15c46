"""GPU octree build vs the oracle and the golden fixtures: keys, permutation, topology, geometry,
moments and quadrupoles bit-exact, including re-key rounds, buckets and the reference's capacity."""

import hashlib

import numpy as np
import pytest

import gen
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TREE_FIELDS = ["Coordinates", "Masses", "Sizes", "Deltas", "Softenings", "Quadrupoles", "FirstSubnode",
               "NextBranch", "TreewalkIndices"]
SMALL_CASES = ["uniform2000q", "plummer3000", "rekey302q", "dup250q", "origin5", "tiny1q", "tiny2q", "tiny3q",
               "lattice216"]


@pytest.fixture(scope="module")
def tg():
    import pytreegrav_gb300 as tg

    return tg


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.dtype.str.encode() + str(a.shape).encode() + a.tobytes()).hexdigest()


def assert_tree_equal(t, ref, quad, label=""):
    assert t.NumParticles == ref.NumParticles
    assert t.NumNodes == ref.NumNodes, f"{label}: capacity {t.NumNodes} vs {ref.NumNodes}"
    assert t.HasCoincidentPoints == ref.HasCoincidentPoints
    for f in TREE_FIELDS:
        if f == "Quadrupoles" and not quad:
            continue
        a, b = getattr(t, f), getattr(ref, f)
        if not np.array_equal(a, b):
            bad = np.argwhere(np.atleast_1d(a != b).reshape(len(a), -1).any(1))[:5].ravel()
            raise AssertionError(f"{label}: {f} differs at rows {bad.tolist()}")


@pytest.mark.parametrize("case", SMALL_CASES)
def test_tree_matches_golden(tg, golden_trees, case):
    g = golden_trees
    quad = bool(g[case + "/quad"])
    import warnings

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        t = tg.ConstructTree(g[case + "/pos"], g[case + "/m"], g[case + "/h"], quadrupole=quad)
    p = case + "/tree/"
    assert t.NumNodes == g[p + "NumNodes"]
    assert t.HasCoincidentPoints == bool(g[p + "HasCoincidentPoints"])
    for f in TREE_FIELDS:
        if f == "Quadrupoles" and not quad:
            continue
        assert np.array_equal(getattr(t, f), g[p + f]), f"{case}: {f}"
    assert np.array_equal(tg.morton_order(g[case + "/pos"]), g[case + "/perm"])


def test_geometric_only_tree(tg, golden_trees):
    g = golden_trees
    t = tg.ConstructTree(g["nomoments500/pos"])
    for f in TREE_FIELDS:
        if f == "Quadrupoles":
            continue
        assert np.array_equal(getattr(t, f), g["nomoments500/tree/" + f]), f


def test_large_tree_digests(tg, golden_bigtree):
    g = golden_bigtree
    s1, s2, s3 = (int(v) for v in g["plummer40k/seeds"])
    x = gen.concentrated(s1, 40000)
    t = tg.ConstructTree(x, gen.masses(s2, 40000), gen.softenings(s3, 40000, 0.01), quadrupole=True)
    p = "plummer40k/serial/"
    assert t.NumNodes == g[p + "NumNodes"]
    for f in TREE_FIELDS:
        assert digest(getattr(t, f)) == str(g[p + f + "__sha256"]), f


@pytest.mark.parametrize("kind,n", [("uniform", 100_000), ("plummer", 1_000_000), ("clustered", 300_000)])
def test_full_size_tree_bit_exact_vs_oracle(tg, kind, n):
    rng = np.random.default_rng(n)
    if kind == "uniform":
        x = rng.random((n, 3))
    elif kind == "plummer":
        u = rng.random(n)
        r = 1 / np.sqrt(u ** (-2 / 3) - 1)
        d = rng.normal(size=(n, 3))
        x = d / np.linalg.norm(d, axis=1)[:, None] * r[:, None]
    else:
        c = rng.uniform(-10, 10, (16, 3))
        x = c[rng.integers(0, 16, n)] + rng.normal(size=(n, 3)) * 0.05
    m = rng.random(n) / n
    h = rng.random(n) * 0.01
    t = tg.ConstructTree(x, m, h, quadrupole=True)
    ref = O.OracleTree(x, m, h, quadrupole=True)
    assert_tree_equal(t, ref, True, kind)


def test_duplicates_and_rekey_paths_vs_oracle(tg):
    rng = np.random.default_rng(3)
    base = rng.random((3000, 3))
    x = np.vstack([base, base[:400], base[:5], 0.25 + 1e-9 * rng.random((200, 3))])
    n = len(x)
    m = rng.random(n) / n
    h = np.full(n, 0.01)
    import warnings

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        t = tg.ConstructTree(x, m, h, quadrupole=True)
    ref = O.OracleTree(x, m, h, quadrupole=True)
    assert t.HasCoincidentPoints
    assert_tree_equal(t, ref, True, "dups")


def test_links_reach_every_particle_once(tg):
    """Fully opening the tree via FirstSubnode/NextBranch visits each particle exactly once."""
    for n in (1, 2, 997, 5000):
        x = np.random.default_rng(n).random((n, 3))
        t = tg.ConstructTree(x, np.full(n, 1.0 / n), np.zeros(n))
        first, nxt, npart = t.FirstSubnode, t.NextBranch, t.NumParticles
        seen, no = [], npart
        for _ in range(4 * t.NumNodes + 16):
            if no <= -1:
                break
            if no < npart:
                seen.append(no)
                no = nxt[no]
            else:
                no = first[no]
        assert np.array_equal(np.sort(seen), np.arange(n))


def test_root_quadrupole_matches_analytic(tg):
    for n in (8, 50, 500, 5000):
        rng = np.random.default_rng(0)
        x, m = rng.random((n, 3)), rng.random(n)
        t = tg.ConstructTree(x, m, np.zeros(n), quadrupole=True)
        root = t.NumParticles
        com = t.Coordinates[root]
        r = x - com
        Qref = 3.0 * np.einsum("i,ik,il->kl", m, r, r) - np.eye(3) * np.sum(m * np.sum(r**2, 1))
        assert np.max(np.abs(t.Quadrupoles[root] - Qref)) / np.max(np.abs(Qref)) < 1e-10


def test_fp64_quadrupoles_on_demand_and_fp32_ones_for_the_walk(tg):
    """The build sums FP32 quadrupoles for the FP32 walk; the FP64 ones (bit-exact, the oracle's)
    come when first asked for: through tg_tree_quadrupoles (device pointer, then also in the tree's
    info) as through copy-out. The FP32 quadrupole walk, which reads the FP32 sums, stays within the
    FP32 walk bar (1e-5 relative RMS) of the FP64 oracle walk over the same groups."""
    import ctypes

    import torch

    from pytreegrav_gb300 import _lib

    rng = np.random.default_rng(4)
    n = 200_000
    x, m, h = rng.normal(size=(n, 3)) ** 3, rng.random(n) / n, np.full(n, 0.01)
    t = tg.ConstructTree(x, m, h, quadrupole=True)
    L = _lib.load()
    info = _lib.TreeInfo()
    _lib.check(L.tg_tree_info_get(t._h, ctypes.byref(info)))
    assert not info.quad  # nothing has needed the FP64 quadrupoles yet
    q = ctypes.c_void_p()
    _lib.check(L.tg_tree_quadrupoles(t._h, ctypes.byref(q), None))
    torch.cuda.synchronize()
    _lib.check(L.tg_tree_info_get(t._h, ctypes.byref(info)))
    assert q.value and info.quad == q.value
    qh = np.empty((t.NumNodes, 3, 3))
    _lib.check(L.tg_tree_copy_out(t._h, None, None, None, None, None, _lib.ptr(qh), None, None, None, None))
    ot = O.OracleTree(x, m, h, quadrupole=True)
    assert np.array_equal(qh, ot.Quadrupoles)
    assert np.array_equal(t.Quadrupoles, ot.Quadrupoles)
    # the FP32 walk with quadrupoles stays at its bar against the FP64 oracle walk
    got = t.fields(accel=True, quadrupole=True, theta=0.7, group_size=8)["accel"]
    idx = ot.TreewalkIndices
    sub = np.arange(0, n, 97)
    inv = np.empty(n, np.int64)
    inv[idx] = np.arange(n)
    pos_s = np.sort(inv[sub])
    starts = np.unique(pos_s // 8 * 8)
    ref = O.fields_groups(ot, x[idx], h[idx], starts, np.minimum(8, n - starts), False, True, False, True, 0.7,
                          nthreads=O.num_threads())["accel"]
    a = got[idx[pos_s]]
    r = ref[pos_s]
    assert np.sqrt(np.mean(np.sum((a - r) ** 2, 1)) / np.mean(np.sum(r**2, 1))) < 1e-5


@pytest.mark.parametrize("where", ["pos", "m", "softening"])
@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_nonfinite_input_raises_like_construct_tree(tg, capsys, where, bad):
    """A NaN or infinity in any input array is found by the device-side check and reported as
    pytreegrav's ConstructTree reports it: the message printed, then RuntimeError (frontend.py:123-125)."""
    rng = np.random.default_rng(5)
    x, m, h = rng.random((300, 3)), np.ones(300), np.full(300, 0.01)
    {"pos": x[:, 2], "m": m, "softening": h}[where][117] = bad
    with pytest.raises(RuntimeError, match="^Invalid input detected - aborting treebuild"):
        tg.ConstructTree(x, m, h)
    assert "Invalid input detected" in capsys.readouterr().out
    with pytest.raises(RuntimeError, match="Invalid input detected"):
        tg.Accel(x, m, h, method="tree")
    # the library is usable right after a rejected call
    x2 = rng.random((300, 3))
    assert np.all(np.isfinite(tg.Accel(x2, np.ones(300), np.full(300, 0.01), method="tree")))


def test_tree_used_on_other_streams_right_after_the_build(tg):
    """A build returns with its moment pass still running on its stream: a walk, a copy-out and a
    column-density call issued at once on other streams must see the finished tree (each entry
    orders its stream after the build), and so give the results of a synchronised build."""
    import ctypes

    import torch

    from pytreegrav_gb300 import _lib

    L = _lib.load()
    vp = ctypes.c_void_p
    rng = np.random.default_rng(12)
    n = 200_000
    x = rng.normal(size=(n, 3))
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.01)
    dx, dm, dh = (torch.from_numpy(a).cuda() for a in (x, m, h))
    ref_tree = tg.ConstructTree(x, m, h, quadrupole=True)
    ref = ref_tree.fields(accel=True, quadrupole=True, group_size=32, grouping="tree")["accel"]
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    for _ in range(3):
        t = vp()
        torch.cuda.synchronize()
        _lib.check(L.tg_tree_build(vp(dx.data_ptr()), vp(dm.data_ptr()), vp(dh.data_ptr()), n, 1, 1,
                                   _lib.TG_MEM_DEVICE, vp(sa.cuda_stream), ctypes.byref(t)), "build")
        out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
        _lib.check(L.tg_tree_fields(t, None, None, n, _lib.TG_FIELD_ACCEL, 1, 0.7, 1.0, 32, _lib.TG_GROUP_TREE,
                                    _lib.TG_ORDER_TREE, _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, vp(out.data_ptr()),
                                    vp(sb.cuda_stream)), "walk")
        info = _lib.TreeInfo()
        _lib.check(L.tg_tree_info_get(t, ctypes.byref(info)))
        mass = np.empty(int(info.num_nodes))
        _lib.check(L.tg_tree_copy_out(t, None, _lib.ptr(mass), None, None, None, None, None, None, None,
                                      vp(sb.cuda_stream)), "copy out")
        sb.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref)
        assert mass[n] == ref_tree.Masses[n]  # the root's mass comes from the moment pass
        L.tg_tree_free(t)
        torch.cuda.synchronize()


def test_trees_share_pooled_streams_and_events(tg):
    """Trees take their side streams and events from the library's pool and return them when freed
    (with work possibly still queued on them): many trees built, walked and freed, two alive at a
    time and freed in either order, give the first tree's results every time."""
    import gc

    from pytreegrav_gb300 import synthetic

    x = synthetic.plummer(20_000, 17)
    n = len(x)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.01)
    kw = dict(accel=True, quadrupole=True, group_size=32, theta=0.7, grouping="tree")
    ref = tg.ConstructTree(x, m, h, quadrupole=True).fields(**kw)["accel"]
    alive = []
    for i in range(24):
        t = tg.ConstructTree(x, m, h, quadrupole=True)
        alive.append(t)
        assert np.array_equal(t.fields(**kw)["accel"], ref), i
        if len(alive) == 2:
            alive.pop(i % 2)  # free the older or the newer one
            gc.collect()
    alive.clear()
    gc.collect()
    assert np.array_equal(tg.ConstructTree(x, m, h, quadrupole=True).fields(**kw)["accel"], ref)
