"""Generate the golden fixtures in tests/golden/ by running pytreegrav's own Python source.

pytreegrav imports numba at module scope and numba is not installed here, so this script puts the
inert stand-in package tests/golden/_numba_shim on sys.path first: decorators become identities and
pytreegrav's unmodified algorithm runs as plain Python (IEEE double, no FMA contraction).

Run from the repository root, with the pytreegrav checkout's src/ directory as the argument:

    python tests/golden/make_golden.py /path/to/pytreegrav/src            (all fixtures)
    python tests/golden/make_golden.py /path/to/pytreegrav/src column     (golden_column.npz only)
    python tests/golden/make_golden.py /path/to/pytreegrav/src corr       (golden_corr.npz only)

Writes tests/golden/golden_*.npz. Small cases store full arrays; large cases store SHA-256 digests of
each array, so the fixtures stay a few hundred KB. Seeds are fixed; rerunning reproduces the files.
"""

import hashlib
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = HERE

TREE_FIELDS = ["Coordinates", "Masses", "Sizes", "Deltas", "Softenings", "Quadrupoles", "FirstSubnode",
               "NextBranch", "TreewalkIndices"]


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.dtype.str.encode() + str(a.shape).encode() + a.tobytes()).hexdigest()


def tree_arrays(tree, prefix, store_full=True):
    d = {}
    d[prefix + "NumParticles"] = np.int64(tree.NumParticles)
    d[prefix + "NumNodes"] = np.int64(tree.NumNodes)
    d[prefix + "HasCoincidentPoints"] = np.bool_(tree.HasCoincidentPoints)
    d[prefix + "HasQuads"] = np.bool_(tree.HasQuads)
    for f in TREE_FIELDS:
        a = getattr(tree, f, None)
        if a is None or (f == "Quadrupoles" and not tree.HasQuads):
            continue
        a = np.asarray(a)
        if store_full:
            d[prefix + f] = a
        else:
            d[prefix + f + "__sha256"] = np.array(digest(a))
    return d


def fingerprint(t):
    """Traversal-order fingerprint (particle visit order + node moments in DFS preorder), as in the
    reference's parallel-vs-serial split test (tests/test_radix_build.py:258-282)."""
    nn = t.NumParticles
    First, Next = np.asarray(t.FirstSubnode), np.asarray(t.NextBranch)
    M, C, D, S = (np.asarray(a) for a in (t.Masses, t.Coordinates, t.Deltas, t.Softenings))
    order, nodes, st = [], [], [nn]
    while st:
        no = st.pop()
        if no < nn:
            order.append(no)
            continue
        nodes.append((M[no], C[no, 0], C[no, 1], C[no, 2], D[no], S[no]))
        kids, c, stop = [], First[no], Next[no]
        while c != -1 and c != stop:
            kids.append(c)
            c = Next[c]
        st.extend(reversed(kids))
    return np.array(order, np.int64), np.array(nodes, np.float64)


def plummer(n, rng):
    u = rng.random(n)
    r = 1.0 / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    d = rng.normal(size=(n, 3))
    return d / np.linalg.norm(d, axis=1)[:, None] * r[:, None]


def main(src):
    sys.path.insert(0, os.path.join(HERE, "_numba_shim"))
    sys.path.insert(0, src)
    warnings.simplefilter("ignore")
    import pytreegrav as pg
    import pytreegrav.octree as om
    from pytreegrav.bruteforce import (Accel_bruteforce_parallel, AccelTarget_bruteforce,
                                       Potential_bruteforce_parallel, PotentialTarget_bruteforce,
                                       TidalTensor_bruteforce_parallel, TidalTensorTarget_bruteforce)
    from pytreegrav.grouped_treewalk import FieldsTarget_grouped, _morton_order
    from pytreegrav.kernel import ForceKernel, PotentialKernel, TidalKernel
    from pytreegrav.octree import _bounding_cube, _morton_keys, _radix_argsort

    # 1. small trees: full arrays -----------------------------------------------------------------
    rng = np.random.default_rng(20251203)
    cases = {}
    cases["uniform2000q"] = (rng.random((2000, 3)), None, 0.01, True)
    x = plummer(3000, rng)
    cases["plummer3000"] = (x, None, "rand", False)
    corners = np.array([[0.0, 0, 0], [1, 1, 1]])
    cases["rekey302q"] = (np.vstack([corners, 0.5 + 1e-8 * rng.random((300, 3))]), None, 1e-3, True)
    b = rng.random((200, 3))
    cases["dup250q"] = (np.vstack([b, b[:50]]), None, 0.02, True)
    cases["origin5"] = (np.array([[0.0, 0, 0], [0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]), None, 0.1, False)
    for n in (1, 2, 3):
        cases[f"tiny{n}q"] = (rng.random((n, 3)), None, 0.1, True)
    lattice = np.arange(6) * 1.0
    cases["lattice216"] = (np.ascontiguousarray(np.stack(np.meshgrid(lattice, lattice, lattice), -1).reshape(-1, 3)),
                           None, 0.1, True)

    tree_out = {}
    for name, (x, m, h, quad) in cases.items():
        n = len(x)
        m = rng.random(n) / n if m is None else m
        h = rng.random(n) * 0.02 if isinstance(h, str) else np.full(n, h)
        t = pg.ConstructTree(x, m, h, quadrupole=quad)
        c, s = _bounding_cube(x)
        keys = _morton_keys(x, c, s)
        tree_out[name + "/pos"] = x
        tree_out[name + "/m"] = m
        tree_out[name + "/h"] = h
        tree_out[name + "/quad"] = np.bool_(quad)
        tree_out[name + "/center"] = c
        tree_out[name + "/size"] = np.float64(s)
        tree_out[name + "/keys"] = keys
        tree_out[name + "/perm"] = _radix_argsort(keys)
        tree_out.update(tree_arrays(t, name + "/tree/"))
    # geometric-only tree (m=None): masses hold only the split's particle folds
    x = rng.random((500, 3))
    t = pg.ConstructTree(x)
    tree_out["nomoments500/pos"] = x
    tree_out.update(tree_arrays(t, "nomoments500/tree/"))
    np.savez_compressed(os.path.join(OUT, "golden_trees.npz"), **tree_out)

    # 2. large trees: digests (serial numbering) + fingerprint of the frontier path ----------------
    big = {}
    sys.path.insert(0, HERE)
    import gen

    # inputs regenerated bit-identically from seeds by tests/golden/gen.py, so only digests are stored
    x = gen.concentrated(101, 40000)
    m = gen.masses(102, 40000)
    h = gen.softenings(103, 40000, 0.01)
    big["plummer40k/seeds"] = np.array([101, 102, 103], np.int64)
    big["plummer40k/pos__sha256"] = np.array(digest(x))
    om.PARALLEL_SPLIT_NMIN = 10**12
    t = pg.ConstructTree(x, m, h, quadrupole=True)
    big.update(tree_arrays(t, "plummer40k/serial/", store_full=False))
    om.PARALLEL_SPLIT_NMIN = 30_000
    tp = pg.ConstructTree(x, m, h, quadrupole=True)
    o_s, n_s = fingerprint(t)
    o_p, n_p = fingerprint(tp)
    assert np.array_equal(o_s, o_p) and np.array_equal(n_s, n_p)
    big["plummer40k/fingerprint_order__sha256"] = np.array(digest(o_p))
    big["plummer40k/fingerprint_nodes__sha256"] = np.array(digest(n_p))
    big["plummer40k/frontier_NumNodes"] = np.int64(tp.NumNodes)
    np.savez_compressed(os.path.join(OUT, "golden_bigtree.npz"), **big)

    # 3. grouped walks, full outputs on group-aligned Morton slices ---------------------------------
    walk = {}
    rng = np.random.default_rng(7)
    x = plummer(3000, rng)
    m = rng.random(3000) / 3000
    h = np.full(3000, 0.05)
    walk["src/pos"], walk["src/m"], walk["src/h"] = x, m, h
    t = pg.ConstructTree(x, m, h, quadrupole=True)
    idx = np.asarray(t.TreewalkIndices)
    xs, hs = x[idx], h[idx]
    for gs in (1, 8, 32):
        for quad in (False, True):
            for theta in (0.4, 0.7):
                sl = slice(0, 256)
                R = FieldsTarget_grouped(xs[sl], hs[sl], t, potential=True, accel=True, tidal=True, group_size=gs,
                                         theta=theta, quadrupole=quad, G=1.0)
                for k, v in R.items():
                    walk[f"g{gs}_q{int(quad)}_t{theta}/{k}"] = v
    # the frontend's own ordering and scatter, end to end
    xf = rng.random((1200, 3))
    mf = np.full(1200, 1 / 1200)
    hf = np.full(1200, 0.01)
    walk["frontend/pos"], walk["frontend/m"], walk["frontend/h"] = xf, mf, hf
    walk["frontend/Accel"] = pg.Accel(xf, mf, hf, method="tree", theta=0.7)
    walk["frontend/Potential"] = pg.Potential(xf, mf, hf, method="tree", theta=0.7, quadrupole=True)
    xt = rng.normal(size=(300, 3)) * 0.6 + 0.5
    ht = np.full(300, 0.005)
    walk["frontend/targets"], walk["frontend/h_t"] = xt, ht
    walk["frontend/AccelTarget"] = pg.AccelTarget(xt, xf, mf, ht, hf, method="tree", theta=0.6)
    walk["frontend/TidalTensorTarget"] = pg.TidalTensorTarget(xt, xf, mf, ht, hf, method="tree", theta=0.6,
                                                              quadrupole=True)
    walk["frontend/morton_order_targets"] = _morton_order(xt)
    np.savez_compressed(os.path.join(OUT, "golden_walk.npz"), **walk)

    # 4. brute force and kernels ----------------------------------------------------------------------
    bf = {}
    rng = np.random.default_rng(11)
    xs_ = rng.normal(size=(400, 3))
    ms_ = rng.random(400) / 400
    hs_ = rng.random(400) * 0.3
    xs_[5] = xs_[4]  # a coincident pair
    xt = np.vstack([rng.normal(size=(60, 3)), xs_[:4]])
    ht = rng.random(64) * 0.1
    bf["src/pos"], bf["src/m"], bf["src/h"], bf["tgt/pos"], bf["tgt/h"] = xs_, ms_, hs_, xt, ht
    bf["PotentialTarget"] = PotentialTarget_bruteforce(xt, ht, xs_, ms_, hs_, G=1.0)
    bf["AccelTarget"] = AccelTarget_bruteforce(xt, ht, xs_, ms_, hs_, G=1.0)
    bf["TidalTensorTarget"] = TidalTensorTarget_bruteforce(xt, ht, xs_, ms_, hs_, G=1.0)
    bf["Potential_mutual"] = Potential_bruteforce_parallel(xs_, ms_, hs_, G=1.0)
    bf["Accel_mutual"] = Accel_bruteforce_parallel(xs_, ms_, hs_, G=1.0)
    bf["TidalTensor_mutual"] = TidalTensor_bruteforce_parallel(xs_, ms_, hs_, G=1.0)
    r = np.concatenate([np.linspace(1e-3, 1.6, 97), [0.5, 1.0]])
    bf["kernel/r"] = r
    bf["kernel/force"] = np.array([ForceKernel(v, 1.0) for v in r])
    bf["kernel/potential"] = np.array([PotentialKernel(v, 1.0) for v in r])
    bf["kernel/tidal"] = np.array([TidalKernel(v, 1.0) for v in r])
    np.savez_compressed(os.path.join(OUT, "golden_bruteforce.npz"), **bf)
    print("wrote", sorted(f for f in os.listdir(OUT) if f.endswith(".npz")))


def column(src):
    """golden_column.npz: pytreegrav's column-density walks (treewalk.py:904-1030) and its
    random_rotation (misc.py:7-55) on a small cloud of uniform spheres."""
    sys.path.insert(0, os.path.join(HERE, "_numba_shim"))
    sys.path.insert(0, src)
    from pytreegrav import ConstructTree
    from pytreegrav.misc import random_rotation
    from pytreegrav.treewalk import ColumnDensityWalk_binned, ColumnDensityWalk_singleray

    rng = np.random.default_rng(17)
    n = 300
    x = rng.normal(size=(n, 3))
    m = rng.random(n) / n
    h = rng.uniform(0.05, 0.5, n)
    h[7] = 0.0  # a point-like particle: no cross-section
    tree = ConstructTree(x, m, h)
    xt = np.vstack([x[:24], rng.normal(size=(16, 3)) * 1.5, [[0.0, 0.0, 0.0], [5.0, 0.0, 0.0]]])
    rays = np.vstack([np.eye(3), -np.eye(3), rng.normal(size=(3, 3))])
    rays /= np.sqrt((rays * rays).sum(1))[:, None]
    col = {"src/pos": x, "src/m": m, "src/h": h, "tgt/pos": xt, "rays": rays}
    col["rays_out"] = np.array([[ColumnDensityWalk_singleray(p, r, tree) for r in rays] for p in xt])
    for theta in (0.5, 0.8):
        col[f"binned_theta{theta}"] = np.array([ColumnDensityWalk_binned(p, tree, theta) for p in xt])
    col["rotations"] = np.array([random_rotation(i) for i in range(12)])
    from pytreegrav.grouped_treewalk import _morton_order
    from pytreegrav.treewalk import ColumnDensityBinned_grouped

    xs = x[_morton_order(x)]  # targets in Morton order, as the frontend passes them
    col["grouped/pos"] = xs
    for gs in (1, 7, 16):
        col[f"binned_grouped_gs{gs}"] = ColumnDensityBinned_grouped(xs, tree, 0.5, gs)
    np.savez_compressed(os.path.join(OUT, "golden_column.npz"), **col)
    print("wrote golden_column.npz")


def corr(src):
    """golden_corr.npz: pytreegrav's DynamicOctree velocity moments (dynamic_tree.py:246-310) and its
    DensityCorrFunc / VelocityCorrFunc / VelocityStructFunc (frontend.py:1047-1320) with
    weighted_binning=True, or with max_bin_size_ratio so small that every particle is binned on its
    own -- the deterministic forms (the default binning jitters with np.random)."""
    sys.path.insert(0, os.path.join(HERE, "_numba_shim"))
    sys.path.insert(0, src)
    warnings.simplefilter("ignore")
    from pytreegrav import ConstructTree, DensityCorrFunc, VelocityCorrFunc, VelocityStructFunc

    rng = np.random.default_rng(23)
    n = 800
    x = plummer(n, rng)
    m = rng.random(n) / n
    v = 0.3 * x + rng.normal(size=(n, 3))  # a bulk flow correlated with position, plus noise
    out = {"pos": x, "m": m, "v": v}
    dt = ConstructTree(x, m, np.zeros(n), vel=v)
    order, nodes = [], []  # DynamicOctree node numbering is its own: store nodes in traversal preorder
    First, Next = np.asarray(dt.FirstSubnode), np.asarray(dt.NextBranch)
    st = [n]
    while st:
        no = st.pop()
        if no < n:
            order.append(no)
            continue
        nodes.append(np.concatenate([[dt.Masses[no]], dt.Coordinates[no], [dt.Sizes[no], dt.Deltas[no]],
                                     dt.Velocities[no], [dt.VelocityDisp[no]]]))
        kids, c, stop = [], First[no], Next[no]
        while c != -1 and c != stop:
            kids.append(c)
            c = Next[c]
        st.extend(reversed(kids))
    out["dyn/order"] = np.array(order, np.int64)
    out["dyn/TreewalkIndices"] = np.asarray(dt.TreewalkIndices)
    out["dyn/nodes_preorder"] = np.array(nodes)  # mass, com(3), size, delta, vel(3), vdisp
    rb, out["density_weighted"] = DensityCorrFunc(x, m, weighted_binning=True)
    out["rbins_default"] = rb
    rb2 = 10 ** np.linspace(-1.5, 1.0, 13)
    out["rbins"] = rb2
    _, out["density_pairs"] = DensityCorrFunc(x, m, rb2, max_bin_size_ratio=1e-300)
    _, out["density_weighted_t0.5"] = DensityCorrFunc(x, m, rb2, theta=0.5, weighted_binning=True)
    _, out["velocity_weighted"] = VelocityCorrFunc(x, m, v, rb2, weighted_binning=True)
    _, out["velocity_pairs"] = VelocityCorrFunc(x, m, v, rb2, max_bin_size_ratio=1e-300)
    _, out["structure_weighted"] = VelocityStructFunc(x, m, v, rb2, weighted_binning=True)
    _, out["structure_weighted_t0.6_mbr3"] = VelocityStructFunc(x, m, v, rb2, theta=0.6, max_bin_size_ratio=3.0,
                                                                weighted_binning=True)
    # periodic box, and targets other than the tree's particles (a supplied tree)
    xu = rng.random((600, 3))
    mu = np.full(600, 1.0 / 600)
    vu = rng.normal(size=(600, 3))
    rb3 = 10 ** np.linspace(-1.7, -0.4, 9)
    out["box/pos"], out["box/m"], out["box/v"], out["box/rbins"] = xu, mu, vu, rb3
    _, out["box/density_weighted"] = DensityCorrFunc(xu, mu, rb3, boxsize=1.0, weighted_binning=True)
    _, out["box/structure_weighted"] = VelocityStructFunc(xu, mu, vu, rb3, boxsize=1.0, weighted_binning=True)
    xt = rng.random((150, 3)) * 2 - 1
    tree = ConstructTree(x, m, np.zeros(n))
    out["targets/pos"] = xt
    _, out["targets/density_weighted"] = DensityCorrFunc(xt, np.ones(150), rb2, tree=tree, weighted_binning=True)
    np.savez_compressed(os.path.join(OUT, "golden_corr.npz"), **out)
    print("wrote golden_corr.npz")


if __name__ == "__main__":
    if len(sys.argv) == 3 and sys.argv[2] == "column":
        column(sys.argv[1])
    elif len(sys.argv) == 3 and sys.argv[2] == "corr":
        corr(sys.argv[1])
    elif len(sys.argv) != 2:
        sys.exit(__doc__)
    else:
        main(sys.argv[1])
        column(sys.argv[1])
        corr(sys.argv[1])
