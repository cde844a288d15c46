"""The batched form on the GPU: many independent systems of uneven size in one segmented build and
one walk, against the same systems built and walked one by one; the walk captured in a CUDA graph;
launch shapes (block shape, first stack) that must not change results; the device-side rewalk of
groups that overflow the small stack; the autotuner."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import pytreegrav_gb300 as tg

    return tg


def systems(n_sys, lo, hi, seed):
    """n_sys systems with N log-uniform in [lo, hi], even ones uniform cubes, odd ones Plummer,
    float32 positions (as the batched configuration), masses 1/N per system."""
    from pytreegrav_gb300 import synthetic

    rng = np.random.default_rng(seed)
    ns = np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), n_sys))).astype(np.int64)
    parts = [(synthetic.uniform(int(k), seed + 7 * s) if s % 2 == 0 else synthetic.plummer(int(k), seed + 7 * s))
             .astype(np.float32).astype(np.float64) for s, k in enumerate(ns)]
    off = np.concatenate([[0], np.cumsum(ns)])
    m = np.concatenate([np.full(k, 1.0 / k) for k in ns])
    return np.vstack(parts), m, off


def rel_rms(a, b):
    return float(np.sqrt(np.mean(np.sum((a - b) ** 2, 1)) / np.mean(np.sum(b ** 2, 1))))


def test_batched_walk_matches_single_systems(tg):
    x, m, off = systems(300, 256, 8192, 1)
    h = np.full(len(x), 0.01)
    tree = tg.Octree.batched(x, m, h, off)
    acc = tree.fields(accel=True, theta=0.7, group_size=32, grouping="tree")["accel"]
    assert np.all(np.isfinite(acc))
    for s in (0, 1, 57, 150, 299):
        a, b = off[s], off[s + 1]
        single = tg.Octree(x[a:b], m[a:b], h[a:b]).fields(accel=True, theta=0.7, group_size=32,
                                                           grouping="tree")["accel"]
        assert rel_rms(acc[a:b], single) <= 1e-6, s
        ref = tg.bruteforce(x[a:b], h[a:b], x[a:b], m[a:b], h[a:b], accel=True, precision="fp64")["accel"]
        assert rel_rms(acc[a:b], ref) < 1e-2, s


def test_graph_replays_equal_the_eager_walk_and_shapes_do_not_matter(tg):
    import torch

    x, m, off = systems(200, 256, 16384, 2)
    h = np.full(len(x), 0.01)
    tree = tg.Octree.batched(x, m, h, off)
    eager = tree.fields(accel=True, theta=0.7, group_size=32, grouping="tree")["accel"]
    for warps, stack in ((2, 1024), (8, 1024), (4, 4096)):
        tree.set_walk_config(warps, stack)
        other = tree.fields(accel=True, theta=0.7, group_size=32, grouping="tree")["accel"]
        assert np.array_equal(other, eager), (warps, stack)
    tree.set_walk_config(4, 1024)
    out = torch.full((len(x), 3), float("nan"), dtype=torch.float64, device="cuda")
    graph = tree.walk_graph(out, accel=True, theta=0.7, group_size=32)
    for _ in range(2):
        graph.launch()
        graph.status()
        assert np.array_equal(out.cpu().numpy(), eager)
        out.fill_(float("nan"))
    graph.close()


def test_groups_that_overflow_the_small_stack_are_rewalked(tg):
    from pytreegrav_gb300 import synthetic

    # two groups of 32 targets spread over the whole box: each group's box holds every node, so no
    # node is accepted and each walk opens the whole tree; deeper trees need deeper stacks
    targets = np.random.default_rng(3).random((64, 3))
    kw = dict(accel=True, theta=0.7, group_size=32, order="given")
    for n in (2_000_000, 8_000_000):
        x = synthetic.uniform(n, 3)
        tree = tg.ConstructTree(x, np.full(n, 1.0 / n), np.full(n, 0.001))
        tree.set_walk_config(4, 1024)
        small = tree.fields(targets, np.zeros(64), **kw)["accel"]
        if tree.last_walk_stats()[2] > 1024:  # a group needed the large stack: the retry pass ran
            break
    else:
        pytest.fail("no walk overflowed the small stack")
    tree.set_walk_config(4, 4096)
    big = tree.fields(targets, np.zeros(64), **kw)["accel"]
    assert np.array_equal(small, big)


def test_autotune_picks_and_applies_a_shape(tg, tmp_path, monkeypatch):
    from pytreegrav_gb300 import autotune

    monkeypatch.setenv("TG_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    x, m, off = systems(64, 256, 16384, 4)
    tree = tg.Octree.batched(x, m, np.full(len(x), 0.01), off)
    res = autotune.tune(tree, n_systems=64, repeats=1)
    assert res["group_size"] in autotune.GROUP_SIZES and res["warps"] in autotune.WARPS
    assert res["stack"] in autotune.STACKS and len(res["timings"]) == 18 and not res["cached"]
    again = autotune.tune(tree, n_systems=64)
    assert again["cached"] and again["warps"] == res["warps"]


def test_full_size_batched_configuration(tg):
    """4096 systems, N log-uniform in [256, 65536] (about 5e7 particles), half uniform, half Plummer,
    float32 positions, h = 0.01, theta = 0.7, monopole: one segmented build, one walk in a CUDA graph."""
    import torch

    x, m, off = systems(4096, 256, 65536, 5)
    h = np.full(len(x), 0.01)
    tree = tg.Octree.batched(x, m, h, off)
    out = torch.empty((len(x), 3), dtype=torch.float64, device="cuda")
    graph = tree.walk_graph(out, accel=True, theta=0.7, group_size=32)
    graph.launch()
    graph.status()
    acc = out.cpu().numpy()
    assert np.all(np.isfinite(acc))
    for s in (3, 1000, 4095):
        a, b = off[s], off[s + 1]
        ref = tg.bruteforce(x[a:b], h[a:b], x[a:b], m[a:b], h[a:b], accel=True, precision="fp32")["accel"]
        assert rel_rms(acc[a:b], ref) < 1e-2, s
    graph.close()
