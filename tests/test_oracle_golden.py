"""The CPU oracle against fixtures generated by running pytreegrav's own Python source.

These pin the oracle before anything is checked against it: Morton keys, the sort permutation, the
whole octree (links, geometry, moments, quadrupoles, capacity) bit-exact; the FP64 grouped walk and
brute force to the last bit, since both evaluate the same expressions in the same order without FMA.
"""

import hashlib

import numpy as np
import pytest

import gen
from oracle import oracle as O

TREE_FIELDS = ["Coordinates", "Masses", "Sizes", "Deltas", "Softenings", "Quadrupoles", "FirstSubnode",
               "NextBranch", "TreewalkIndices"]
SMALL_CASES = ["uniform2000q", "plummer3000", "rekey302q", "dup250q", "origin5", "tiny1q", "tiny2q", "tiny3q",
               "lattice216"]


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.dtype.str.encode() + str(a.shape).encode() + a.tobytes()).hexdigest()


@pytest.mark.parametrize("case", SMALL_CASES)
def test_keys_and_permutation_bit_exact(golden_trees, case):
    g = golden_trees
    pos = g[case + "/pos"]
    c, s = O.bounding_cube(pos)
    assert np.array_equal(c, g[case + "/center"]) and s == g[case + "/size"]
    keys = O.morton_keys(pos, c, s)
    assert np.array_equal(keys, g[case + "/keys"])
    perm = O.radix_argsort(keys)
    assert np.array_equal(perm, g[case + "/perm"])
    assert np.array_equal(perm, np.argsort(keys, kind="stable"))


@pytest.mark.parametrize("case", SMALL_CASES)
def test_tree_bit_exact(golden_trees, case):
    g = golden_trees
    quad = bool(g[case + "/quad"])
    t = O.OracleTree(g[case + "/pos"], g[case + "/m"], g[case + "/h"], quadrupole=quad)
    p = case + "/tree/"
    assert t.NumParticles == g[p + "NumParticles"]
    assert t.NumNodes == g[p + "NumNodes"]
    assert t.HasCoincidentPoints == bool(g[p + "HasCoincidentPoints"])
    for f in TREE_FIELDS:
        if f == "Quadrupoles" and not quad:
            continue
        assert np.array_equal(getattr(t, f), g[p + f]), f"{case}: {f} differs"


def test_geometric_only_tree(golden_trees):
    g = golden_trees
    t = O.OracleTree(g["nomoments500/pos"], None, None)
    for f in TREE_FIELDS:
        if f == "Quadrupoles":
            continue
        assert np.array_equal(getattr(t, f), g["nomoments500/tree/" + f]), f


def test_large_tree_serial_numbering_digests(golden_bigtree):
    g = golden_bigtree
    s1, s2, s3 = (int(v) for v in g["plummer40k/seeds"])
    x = gen.concentrated(s1, 40000)
    assert digest(x) == str(g["plummer40k/pos__sha256"]), "fixture input generator drifted"
    t = O.OracleTree(x, gen.masses(s2, 40000), gen.softenings(s3, 40000, 0.01), quadrupole=True)
    p = "plummer40k/serial/"
    assert t.NumNodes == g[p + "NumNodes"]
    for f in TREE_FIELDS:
        assert digest(getattr(t, f)) == str(g[p + f + "__sha256"]), f


@pytest.mark.parametrize("gs", [1, 8, 32])
@pytest.mark.parametrize("quad", [False, True])
@pytest.mark.parametrize("theta", [0.4, 0.7])
def test_grouped_walk_bit_exact(golden_walk, gs, quad, theta):
    g = golden_walk
    t = O.OracleTree(g["src/pos"], g["src/m"], g["src/h"], quadrupole=True)
    idx = t.TreewalkIndices
    xs, hs = g["src/pos"][idx][:256], g["src/h"][idx][:256]
    res = t.fields(xs, hs, True, True, True, quad, gs, theta)
    for k in ("potential", "accel", "tidal"):
        assert np.array_equal(res[k], g[f"g{gs}_q{int(quad)}_t{theta}/{k}"]), k


def test_frontend_ordering(golden_walk):
    g = golden_walk
    x, m, h = g["frontend/pos"], g["frontend/m"], g["frontend/h"]
    a, _ = O.self_fields(x, m, h, accel=True, theta=0.7)
    assert np.array_equal(a["accel"], g["frontend/Accel"])
    p, _ = O.self_fields(x, m, h, potential=True, theta=0.7, quadrupole=True)
    assert np.array_equal(p["potential"], g["frontend/Potential"])
    xt, ht = g["frontend/targets"], g["frontend/h_t"]
    assert np.array_equal(O.morton_order(xt), g["frontend/morton_order_targets"])
    at, _ = O.target_fields(xt, ht, x, m, h, accel=True, theta=0.6)
    assert np.array_equal(at["accel"], g["frontend/AccelTarget"])
    tt, _ = O.target_fields(xt, ht, x, m, h, tidal=True, theta=0.6, quadrupole=True)
    assert np.array_equal(tt["tidal"], g["frontend/TidalTensorTarget"])


def test_bruteforce_bit_exact(golden_bruteforce):
    g = golden_bruteforce
    xs, ms, hs, xt, ht = g["src/pos"], g["src/m"], g["src/h"], g["tgt/pos"], g["tgt/h"]
    r = O.bruteforce(xt, ht, xs, ms, hs, True, True, True)
    assert np.array_equal(r["potential"], g["PotentialTarget"])
    assert np.array_equal(r["accel"], g["AccelTarget"])
    assert np.array_equal(r["tidal"], g["TidalTensorTarget"])
    r = O.bruteforce(xs, hs, xs, ms, hs, True, True, True, mutual=True)
    assert np.array_equal(r["potential"], g["Potential_mutual"])
    assert np.array_equal(r["accel"], g["Accel_mutual"])
    assert np.array_equal(r["tidal"], g["TidalTensor_mutual"])


def test_kernels_bit_exact(golden_bruteforce):
    g = golden_bruteforce
    for v, f, p, t in zip(g["kernel/r"], g["kernel/force"], g["kernel/potential"], g["kernel/tidal"]):
        assert O.force_kernel(v, 1.0) == f
        assert O.potential_kernel(v, 1.0) == p
        assert O.tidal_kernel(v, 1.0) == t


def test_oracle_thread_count_independence(golden_walk):
    """OpenMP splits groups across threads; each group accumulates privately, so results match."""
    g = golden_walk
    t = O.OracleTree(g["src/pos"], g["src/m"], g["src/h"], quadrupole=True)
    idx = t.TreewalkIndices
    xs, hs = g["src/pos"][idx], g["src/h"][idx]
    a = t.fields(xs, hs, True, True, False, True, 8, 0.5, nthreads=1)
    b = t.fields(xs, hs, True, True, False, True, 8, 0.5, nthreads=4)
    for k in a:
        assert np.array_equal(a[k], b[k])


def test_column_density_walks_bit_exact(golden_column):
    """The oracle's ray-traced and angle-binned column-density walks against pytreegrav's own
    (treewalk.py:904-1030), run on the same tree: identical to the last bit."""
    g = golden_column
    t = O.OracleTree(g["src/pos"], g["src/m"], g["src/h"])
    got = O.column_rays(t, g["tgt/pos"], g["rays"])
    assert np.array_equal(got, g["rays_out"])
    for theta in (0.5, 0.8):
        assert np.array_equal(O.column_binned(t, g["tgt/pos"], theta), g[f"binned_theta{theta}"])
    # per-target ray sets: the same rays repeated per target give the same columns
    per = np.broadcast_to(g["rays"], (len(g["tgt/pos"]),) + g["rays"].shape)
    assert np.array_equal(O.column_rays(t, g["tgt/pos"], per, per_target=True), g["rays_out"])


def test_grouped_binned_column_density_bit_exact(golden_column):
    g = golden_column
    t = O.OracleTree(g["src/pos"], g["src/m"], g["src/h"])
    for gs in (1, 7, 16):
        assert np.array_equal(O.column_binned_grouped(t, g["grouped/pos"], 0.5, gs), g[f"binned_grouped_gs{gs}"]), gs
