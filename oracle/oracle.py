"""Python face of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads oracle/_build/libtg_oracle.so (built by oracle/build_oracle.py) and reproduces pytreegrav's
frontend ordering on top of it: self-gravity targets go in the tree's TreewalkIndices order,
external targets (and self-gravity against a supplied tree) in their own Morton order, and results
are scattered back to the caller's order (src/pytreegrav/frontend.py:244-288, 392-416, 514-555,
659-680). Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""

import ctypes
import os

import numpy as np

from . import build_oracle

_LIB = None
_i64 = ctypes.c_int64
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int64)


class _Tree(ctypes.Structure):
    _fields_ = [
        ("npart", _i64),
        ("num_nodes", _i64),
        ("node_hi", _i64),
        ("has_quads", ctypes.c_int),
        ("has_coincident", ctypes.c_int),
        ("coord", _dp),
        ("mass", _dp),
        ("size", _dp),
        ("delta", _dp),
        ("soft", _dp),
        ("quad", _dp),
        ("first", _ip),
        ("next", _ip),
        ("walk_idx", _ip),
    ]


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        L.tgo_build.argtypes = [_dp, _dp, _dp, _i64, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_Tree)]
        L.tgo_free.argtypes = [ctypes.POINTER(_Tree)]
        L.tgo_fields.argtypes = [ctypes.POINTER(_Tree), _dp, _dp, _i64, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, _i64, ctypes.c_double, ctypes.c_double,
                                 _dp, ctypes.c_int]
        L.tgo_walk_counts.argtypes = [ctypes.POINTER(_Tree), _dp, _dp, _i64, _i64, ctypes.c_double,
                                      _ip, _ip, ctypes.c_int]
        L.tgo_walk_counts_groups.argtypes = [ctypes.POINTER(_Tree), _dp, _dp, _ip, _ip, _i64, ctypes.c_double,
                                             _ip, _ip, ctypes.c_int]
        L.tgo_fields_groups.argtypes = [ctypes.POINTER(_Tree), _dp, _dp, _ip, _ip, _i64, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, _dp, ctypes.c_int]
        L.tgo_bruteforce.argtypes = [_dp, _dp, _i64, _dp, _dp, _dp, _i64, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp, ctypes.c_int]
        L.tgo_morton_keys.argtypes = [_dp, _i64, _dp, ctypes.c_double, _ip]
        L.tgo_radix_argsort.argtypes = [_ip, _i64, _ip]
        L.tgo_morton_order.argtypes = [_dp, _i64, _ip]
        L.tgo_bounding_cube.argtypes = [_dp, _i64, _dp, _dp]
        L.tgo_column_rays.argtypes = [ctypes.POINTER(_Tree), _dp, _i64, _dp, _i64, _i64, _dp, ctypes.c_int]
        L.tgo_column_binned.argtypes = [ctypes.POINTER(_Tree), _dp, _i64, ctypes.c_double, _dp, ctypes.c_int]
        L.tgo_column_binned_grouped.argtypes = [ctypes.POINTER(_Tree), _dp, _i64, ctypes.c_double, _i64, _dp,
                                                ctypes.c_int]
        L.tgo_tree_velocities.argtypes = [ctypes.POINTER(_Tree), _dp, _dp, _dp]
        L.tgo_corr_uniform.argtypes = [ctypes.c_uint64, _i64, _i64]
        L.tgo_corr_uniform.restype = ctypes.c_double
        L.tgo_correlation.argtypes = [ctypes.POINTER(_Tree), _dp, _dp, ctypes.c_int, _dp, _dp, _dp, _i64, _dp,
                                      ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_uint64, ctypes.c_int, _dp, _dp, ctypes.c_int]
        for k in ("tgo_force_kernel", "tgo_potential_kernel", "tgo_tidal_kernel"):
            getattr(L, k).argtypes = [ctypes.c_double, ctypes.c_double]
            getattr(L, k).restype = ctypes.c_double
        _LIB = L
    return _LIB


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _f64c(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        a = a.reshape(shape)
    return a


def bounding_cube(pos):
    pos = _f64c(pos, (-1, 3))
    c = np.zeros(3)
    s = np.zeros(1)
    lib().tgo_bounding_cube(_d(pos), len(pos), _d(c), _d(s))
    return c, float(s[0])


def morton_keys(pos, center, size):
    pos = _f64c(pos, (-1, 3))
    c = _f64c(center)
    k = np.empty(len(pos), np.int64)
    lib().tgo_morton_keys(_d(pos), len(pos), _d(c), float(size), _i(k))
    return k


def radix_argsort(keys):
    keys = np.ascontiguousarray(keys, dtype=np.int64)
    p = np.empty(len(keys), np.int64)
    lib().tgo_radix_argsort(_i(keys), len(keys), _i(p))
    return p


def morton_order(pos):
    pos = _f64c(pos, (-1, 3))
    p = np.empty(len(pos), np.int64)
    if len(pos):
        lib().tgo_morton_order(_d(pos), len(pos), _i(p))
    return p


class OracleTree:
    """Host copy of the oracle's octree, with pytreegrav's Octree attribute names."""

    def __init__(self, pos, m=None, softening=None, quadrupole=False, compute_moments=True):
        pos = _f64c(pos, (-1, 3))
        n = len(pos)
        mm = None if m is None else _f64c(m, (n,))
        hh = np.zeros(n) if softening is None else _f64c(softening, (n,))
        t = _Tree()
        rc = lib().tgo_build(_d(pos), None if mm is None else _d(mm), _d(hh), n, int(quadrupole),
                             int(compute_moments), ctypes.byref(t))
        if rc:
            raise RuntimeError(f"oracle build failed ({rc})")
        self._t = t
        nn = t.num_nodes
        self.NumParticles = t.npart
        self.NumNodes = nn
        self.node_hi = t.node_hi
        self.HasQuads = bool(t.has_quads)
        self.HasCoincidentPoints = bool(t.has_coincident)
        self.Coordinates = np.ctypeslib.as_array(t.coord, (nn, 3)).copy()
        self.Masses = np.ctypeslib.as_array(t.mass, (nn,)).copy()
        self.Sizes = np.ctypeslib.as_array(t.size, (nn,)).copy()
        self.Deltas = np.ctypeslib.as_array(t.delta, (nn,)).copy()
        self.Softenings = np.ctypeslib.as_array(t.soft, (nn,)).copy()
        self.Quadrupoles = np.ctypeslib.as_array(t.quad, (nn, 3, 3)).copy() if t.has_quads else None
        self.FirstSubnode = np.ctypeslib.as_array(t.first, (nn,)).copy()
        self.NextBranch = np.ctypeslib.as_array(t.next, (nn,)).copy()
        self.TreewalkIndices = np.ctypeslib.as_array(t.walk_idx, (n,)).copy()

    def __del__(self):
        try:
            lib().tgo_free(ctypes.byref(self._t))
        except Exception:
            pass

    def fields(self, pos, soft, potential=False, accel=False, tidal=False, quadrupole=False,
               group_size=8, theta=0.7, G=1.0, nthreads=0):
        """FieldsTarget_grouped on targets already in the order to be grouped."""
        pos = _f64c(pos, (-1, 3))
        soft = _f64c(soft, (len(pos),))
        W = int(potential) + 3 * int(accel) + 9 * int(tidal)
        out = np.zeros((len(pos), W))
        rc = lib().tgo_fields(ctypes.byref(self._t), _d(pos), _d(soft), len(pos), int(potential),
                              int(accel), int(tidal), int(quadrupole), int(group_size), float(theta),
                              float(G), _d(out), int(nthreads))
        if rc:
            raise ValueError(f"oracle walk failed ({rc})")
        res, o = {}, 0
        if potential:
            res["potential"] = out[:, 0].copy()
            o = 1
        if accel:
            res["accel"] = out[:, o:o + 3].copy()
            o += 3
        if tidal:
            res["tidal"] = out[:, o:o + 9].reshape(-1, 3, 3).copy()
        return res

    def walk_counts(self, pos, soft, group_size=8, theta=0.7, nthreads=0):
        pos = _f64c(pos, (-1, 3))
        soft = _f64c(soft, (len(pos),))
        ng = (len(pos) + group_size - 1) // group_size
        ni = np.zeros(ng, np.int64)
        no = np.zeros(ng, np.int64)
        lib().tgo_walk_counts(ctypes.byref(self._t), _d(pos), _d(soft), len(pos), int(group_size),
                              float(theta), _i(ni), _i(no), int(nthreads))
        return ni, no


def fields_groups(tree, pos, soft, starts, counts, potential=False, accel=False, tidal=False, quadrupole=False,
                  theta=0.7, G=1.0, nthreads=0):
    """FP64 grouped walk over explicitly given groups; pos/soft in walk order, out in that order."""
    pos = _f64c(pos, (-1, 3))
    soft = _f64c(soft, (len(pos),))
    starts = np.ascontiguousarray(starts, np.int64)
    counts = np.ascontiguousarray(counts, np.int64)
    W = int(potential) + 3 * int(accel) + 9 * int(tidal)
    out = np.zeros((len(pos), W))
    rc = lib().tgo_fields_groups(ctypes.byref(tree._t), _d(pos), _d(soft), _i(starts), _i(counts), len(starts),
                                 int(potential), int(accel), int(tidal), int(quadrupole), float(theta), float(G),
                                 _d(out), int(nthreads))
    if rc:
        raise ValueError(f"oracle walk failed ({rc})")
    res, o = {}, 0
    if potential:
        res["potential"] = out[:, 0].copy()
        o = 1
    if accel:
        res["accel"] = out[:, o:o + 3].copy()
        o += 3
    if tidal:
        res["tidal"] = out[:, o:o + 9].reshape(-1, 3, 3).copy()
    return res


def tree_groups(tree, G=32):
    """The engine's tree grouping restated: subtrees and runs of siblings of at most G particles,
    a run never reaching into a large sibling's cell. Returns (starts, counts) in Morton order."""
    N, node_hi = tree.NumParticles, tree.node_hi
    first, nxt = tree.FirstSubnode, tree.NextBranch
    pos = tree.Coordinates[:N]
    size = tree.Sizes
    geo = OracleTree(pos, None, None).Coordinates  # geometric cell centres, same topology

    def children(f):
        c, out = first[f], []
        while c != nxt[f] and c >= 0:
            out.append(c)
            c = nxt[c]
        return out

    lo = np.zeros(node_hi, np.int64)
    hi = np.zeros(node_hi, np.int64)
    for f in range(node_hi - 1, N - 1, -1):
        ch = children(f)
        lo[f] = min(c if c < N else lo[c] for c in ch)
        hi[f] = max(c + 1 if c < N else hi[c] for c in ch)
    S, C = [], []
    for f in range(N, node_hi):
        if hi[f] - lo[f] <= G:
            if f == N:
                S.append(lo[f]); C.append(hi[f] - lo[f])
            continue
        ch = children(f)
        big = [(geo[c] - 0.5 * size[c], geo[c] + 0.5 * size[c]) for c in ch if c >= N and hi[c] - lo[c] > G]
        run_lo, run, rb = -1, 0, None
        for c in ch:
            l, h = (c, c + 1) if c < N else (lo[c], hi[c])
            if h - l > G:
                if run:
                    S.append(run_lo); C.append(run)
                run = 0
                continue
            b = (pos[l:h].min(0), pos[l:h].max(0))
            if run:
                nb = (np.minimum(rb[0], b[0]), np.maximum(rb[1], b[1]))
                hits = any(np.all(nb[0] <= B[1]) and np.all(nb[1] >= B[0]) for B in big)
                if run + (h - l) <= G and not hits:
                    run += h - l
                    rb = nb
                    continue
                S.append(run_lo); C.append(run)
            run_lo, run, rb = l, h - l, b
        if run:
            S.append(run_lo); C.append(run)
    S, C = np.array(S, np.int64), np.array(C, np.int64)
    o = np.argsort(S)
    return S[o], C[o]


def walk_counts_groups(tree, pos, soft, starts, counts, theta=0.7, nthreads=0):
    """Interactions and opened nodes per explicitly given group (pos/soft in walk order)."""
    pos = _f64c(pos, (-1, 3))
    soft = _f64c(soft, (len(pos),))
    starts = np.ascontiguousarray(starts, np.int64)
    counts = np.ascontiguousarray(counts, np.int64)
    ni = np.zeros(len(starts), np.int64)
    no = np.zeros(len(starts), np.int64)
    lib().tgo_walk_counts_groups(ctypes.byref(tree._t), _d(pos), _d(soft), _i(starts), _i(counts), len(starts),
                                 float(theta), _i(ni), _i(no), int(nthreads))
    return ni, no


def bruteforce(pos_t, h_t, pos_s, m_s, h_s, potential=False, accel=False, tidal=False, mutual=False,
               G=1.0, nthreads=0):
    pos_t = _f64c(pos_t, (-1, 3))
    pos_s = _f64c(pos_s, (-1, 3))
    h_t = np.zeros(len(pos_t)) if h_t is None else _f64c(h_t, (len(pos_t),))
    h_s = np.zeros(len(pos_s)) if h_s is None else _f64c(h_s, (len(pos_s),))
    m_s = _f64c(m_s, (len(pos_s),))
    W = int(potential) + 3 * int(accel) + 9 * int(tidal)
    out = np.zeros((len(pos_t), W))
    lib().tgo_bruteforce(_d(pos_t), _d(h_t), len(pos_t), _d(pos_s), _d(m_s), _d(h_s), len(pos_s),
                         int(potential), int(accel), int(tidal), int(mutual), float(G), _d(out),
                         int(nthreads))
    res, o = {}, 0
    if potential:
        res["potential"] = out[:, 0].copy()
        o = 1
    if accel:
        res["accel"] = out[:, o:o + 3].copy()
        o += 3
    if tidal:
        res["tidal"] = out[:, o:o + 9].reshape(-1, 3, 3).copy()
    return res


def self_fields(pos, m, h, potential=False, accel=False, tidal=False, theta=0.7, quadrupole=False,
                group_size=8, G=1.0, tree=None, nthreads=0):
    """Potential/Accel/TidalTensor(method='tree') semantics (frontend.py:244-288)."""
    pos = _f64c(pos, (-1, 3))
    h = np.zeros(len(pos)) if h is None else _f64c(h, (len(pos),))
    if tree is None:
        tree = OracleTree(pos, m, h, quadrupole=quadrupole)
        idx = tree.TreewalkIndices
    else:
        idx = morton_order(pos)
    res = tree.fields(pos[idx], h[idx], potential, accel, tidal, quadrupole, group_size, theta, G,
                      nthreads)
    out = {}
    for k, v in res.items():
        o = np.empty_like(v)
        o[idx] = v
        out[k] = o
    return out, tree


def target_fields(pos_t, h_t, pos_s, m_s, h_s, potential=False, accel=False, tidal=False, theta=0.7,
                  quadrupole=False, group_size=8, G=1.0, tree=None, nthreads=0):
    """PotentialTarget/AccelTarget/TidalTensorTarget(method='tree') semantics (frontend.py:392-416)."""
    pos_t = _f64c(pos_t, (-1, 3))
    h_t = np.zeros(len(pos_t)) if h_t is None else _f64c(h_t, (len(pos_t),))
    if tree is None:
        tree = OracleTree(pos_s, m_s, h_s, quadrupole=quadrupole)
    ts = morton_order(pos_t)
    res = tree.fields(pos_t[ts], h_t[ts], potential, accel, tidal, quadrupole, group_size, theta, G,
                      nthreads)
    out = {}
    for k, v in res.items():
        o = np.empty_like(v)
        o[ts] = v
        out[k] = o
    return out, tree


def column_rays(tree, pos, rays, per_target=False, nthreads=0):
    """Ray-traced column density (treewalk.py:904-973) of every (target, ray): rays (nrays, 3) shared
    by all targets, or (n, nrays, 3) with per_target. Returns (n, nrays)."""
    pos = _f64c(pos, (-1, 3))
    n = len(pos)
    rays = np.ascontiguousarray(rays, np.float64)
    nrays = rays.shape[-2] if rays.ndim == 3 else rays.shape[0]
    stride = 3 * nrays if per_target else 0
    out = np.zeros((n, nrays))
    lib().tgo_column_rays(ctypes.byref(tree._t), _d(pos), n, _d(rays), nrays, stride, _d(out), int(nthreads))
    return out


def column_binned(tree, pos, theta=0.5, nthreads=0):
    """Angle-binned column density (treewalk.py:976-1030), (n, 6)."""
    pos = _f64c(pos, (-1, 3))
    out = np.zeros((len(pos), 6))
    lib().tgo_column_binned(ctypes.byref(tree._t), _d(pos), len(pos), float(theta), _d(out), int(nthreads))
    return out


def column_binned_grouped(tree, pos, theta=0.5, group_size=16, nthreads=0):
    """ColumnDensityBinned_grouped (treewalk.py:1197-1294): targets in the order to be grouped, (n, 6)."""
    pos = _f64c(pos, (-1, 3))
    out = np.zeros((len(pos), 6))
    lib().tgo_column_binned_grouped(ctypes.byref(tree._t), _d(pos), len(pos), float(theta), int(group_size),
                                    _d(out), int(nthreads))
    return out


def tree_velocities(tree, vel):
    """Node velocities and dispersions of pytreegrav's DynamicOctree (dynamic_tree.py:246-310) on the
    oracle tree: (NumNodes, 3) and (NumNodes,), particles in tree order."""
    vel = _f64c(vel, (-1, 3))
    v = np.zeros((tree.NumNodes, 3))
    d = np.zeros(tree.NumNodes)
    lib().tgo_tree_velocities(ctypes.byref(tree._t), _d(vel), _d(v), _d(d))
    return v, d


CORR_KINDS = {"density": 0, "velocity": 1, "structure": 2}


def correlation(tree, kind, pos, rbins, vel=None, weight=None, tree_vel=None, max_bin_size_ratio=100, theta=1.0,
                boxsize=0.0, weighted_binning=False, seed=0, absval=False, nthreads=0):
    """The density (treewalk.py:378-510), velocity-correlation (515-663) or structure-function
    (668-818) walk of every target in pos, summed over targets: (binsums, wtsums). tree_vel is
    tree_velocities(tree, v) for the velocity kinds. absval sums |contribution| instead."""
    k = CORR_KINDS[kind]
    pos = _f64c(pos, (-1, 3))
    n = len(pos)
    rbins = _f64c(rbins)
    nb = len(rbins) - 1
    bs, ws = np.zeros(nb), np.zeros(nb)
    args = [None, None, None, None]
    if k:
        tv, td = tree_vel
        args = [_f64c(tv), _f64c(td), _f64c(vel, (n, 3)), _f64c(weight, (n,))]
    keep = args
    rc = lib().tgo_correlation(ctypes.byref(tree._t), *(None if a is None else _d(a) for a in keep[:2]), k, _d(pos),
                               *(None if a is None else _d(a) for a in keep[2:]), n, _d(rbins), nb,
                               float(max_bin_size_ratio), float(theta), float(boxsize), int(bool(weighted_binning)),
                               int(seed) & (2**64 - 1), int(bool(absval)), _d(bs), _d(ws), int(nthreads))
    if rc:
        raise RuntimeError(f"oracle correlation failed ({rc})")
    return bs, ws


def corr_uniform(seed, target, draw):
    return lib().tgo_corr_uniform(int(seed) & (2**64 - 1), int(target), int(draw))


def force_kernel(r, h):
    return lib().tgo_force_kernel(float(r), float(h))


def potential_kernel(r, h):
    return lib().tgo_potential_kernel(float(r), float(h))


def tidal_kernel(r, h):
    return lib().tgo_tidal_kernel(float(r), float(h))


def num_threads():
    return os.cpu_count() or 1
