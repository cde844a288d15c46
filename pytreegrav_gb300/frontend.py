"""pytreegrav's public gravity API (src/pytreegrav/frontend.py) on the GB300 engine.

Same function names, arguments, defaults, return shapes, ordering and exceptions as pytreegrav's
tree and brute-force paths; every computation runs on the GPU through libpytreegrav_gb300.

Differences a caller can see, all deliberate:
  * ``parallel`` is accepted and ignored: the GPU path is always parallel, and results do not
    depend on it (pytreegrav's own parallel and serial walks are bit-identical too).
  * ``precision`` (keyword, extension): the tree walk evaluates interactions in FP32 with
    compensated accumulation by default ("fp32"); "fp64" evaluates them in FP64. Either way the
    tree (keys, topology, moments) is bit-identical to pytreegrav's and the accepted node set is
    pytreegrav's exactly. Brute force defaults to FP64 (bit-identical sums) for device="cpu" and
    FP32 for device="cuda", matching what each device meant in pytreegrav.
  * ``grouping`` (keyword, extension): "blocks" (default) groups ``group_size`` consecutive
    Morton-ordered targets per traversal, pytreegrav's grouping, so the accepted node set is
    pytreegrav's exactly; "tree" takes groups of at most ``group_size`` particles from a tree -- the
    freshly built tree itself for self-gravity, or an octree of the external targets -- which never
    straddle a jump of the Morton curve: the engine's fast path.
  * ``learned`` / ``error_ratio`` (keywords, extension; every field function and Field):
    ``learned=True`` lets the packaged network set each group's acceptance test (a mass-aware
    tolerance per group, trained on the GPU against brute force) instead of one global theta;
    ``error_ratio`` asks for that RMS force error relative to the plain walk at theta = 0.7. See
    ``pytreegrav_gb300.theta``. With external targets (the *Target forms, or a given tree), the
    targets are grouped by an octree of their own (``TargetSet``), as with ``grouping="tree"``.
  * ``morton_order=False``/``radix=False`` in ConstructTree still build the radix tree (pytreegrav
    documents both builds as giving identical fields on generic data); with ``vel`` the radix tree
    carries the DynamicOctree's node velocities and dispersions.
  * The correlation functions' default binning jitters a node's distance with a counter-based
    generator keyed by ``seed`` (keyword, extension; None draws it from numpy's global generator)
    instead of numba's np.random stream, and clamps a jittered bin index into range.
"""

import warnings

import numpy as np
from numpy import zeros

from . import _lib
from .tree import Octree, bruteforce, morton_order

SYMMETRIC_NMIN = 1000


def _f64(a):
    """Cast to float64 without collapsing a length-1 array to a scalar (frontend.py:20-25)."""
    return np.asarray(a, dtype=np.float64)


def checkTreeQuadrupoles(tree, quadrupole):
    """Raise ValueError if a quadrupole treewalk is requested on a tree that lacks them."""
    if quadrupole and not tree.HasQuads:
        raise ValueError(
            "quadrupole=True requires a tree built with quadrupole moments: pass a tree from "
            "ConstructTree(..., quadrupole=True), or evaluate with quadrupole=False.")


def valueTestMethod(method):
    """Raise TypeError/ValueError unless method is one of 'adaptive', 'bruteforce', 'tree'."""
    methods = ["adaptive", "bruteforce", "tree"]
    if type(method) != str:
        raise TypeError("Invalid method type %s, must be str" % type(method))
    if method not in methods:
        raise ValueError("Invalid method %s. Must be one of: %s" % (method, str(methods)))


def warn_if_coincident_positions(tree, softening=None):
    """Warn if the build found particle positions coincident to floating-point precision."""
    if not tree.HasCoincidentPoints:
        return
    if softening is not None and np.any(softening > 0):
        warnings.warn("Warning: Particle positions are non-unique. Softening will determine the answer for "
                      "overlapping particles.")
        return
    warnings.warn("Warning: Particle positions are non-unique. The answer will be singular or garbage for "
                  "overlapping particles.")


def _check_device(device, quadrupole):
    if device not in ("cpu", "cuda"):
        raise ValueError(f"device must be 'cpu' or 'cuda', got {device!r}")
    if device == "cuda" and quadrupole:
        raise ValueError("device='cuda' is monopole only; pass quadrupole=False")


def _bf_precision(device):
    return "fp32" if device == "cuda" else "fp64"


def _check_tree(tree):
    if not isinstance(tree, Octree):
        raise TypeError("tree must be an Octree built by pytreegrav_gb300.ConstructTree")


def ConstructTree(pos, m=None, softening=None, quadrupole=False, vel=None, compute_moments=True, morton_order=True,
                  radix=True):
    """Build a tree of the particle data on the GPU for subsequent field evaluation.

    Same arguments as pytreegrav.ConstructTree (frontend.py:73-142). Returns an Octree whose arrays
    are bit-identical to pytreegrav's radix build. With vel, the tree also carries the velocities
    and velocity dispersions of pytreegrav's DynamicOctree (Velocities, VelocityDisp): that
    insertion-built tree has the radix tree's topology and traversal order on inputs without
    coincident points, and its moments agree to rounding, so the velocities are attached to this
    tree rather than to a second one.
    """
    pos = np.atleast_2d(_f64(pos))
    if m is None:
        compute_moments = False
    else:
        m = np.atleast_1d(_f64(m))
    if softening is None:
        softening = zeros(len(pos))
    softening = np.atleast_1d(_f64(softening))
    # non-finite positions, masses or softenings are found by the library's device-side check
    # (TG_ERR_NONFINITE), which frontend.py:123-125's print-and-raise then reports
    try:
        tree = Octree(pos, m, softening, quadrupole=quadrupole, compute_moments=compute_moments)
    except _lib.NonFiniteInput:
        print(_lib.NONFINITE_MSG)
        raise RuntimeError(_lib.NONFINITE_MSG) from None
    if vel is not None:
        tree.set_velocities(np.atleast_2d(_f64(vel)))
    warn_if_coincident_positions(tree, softening)
    return tree


def _self_field(key, pos, m, softening, G, theta, tree, return_tree, method, quadrupole, group_size, device,
                precision, parallel_threshold, grouping="blocks", learned=None, error_ratio=None):
    valueTestMethod(method)
    pos = np.atleast_2d(_f64(pos))
    m = np.atleast_1d(_f64(m))
    if softening is None:
        softening = np.zeros_like(m)
    softening = np.atleast_1d(_f64(softening))
    if method == "adaptive":
        method = "tree" if (tree is not None or len(pos) > parallel_threshold) else "bruteforce"
    if device is not None:
        _check_device(device, quadrupole)
    if method == "bruteforce":
        res = bruteforce(None, None, pos, m, softening, mutual=True, G=G, precision=_bf_precision(device),
                         **{key: True})[key]
        if return_tree:
            tree = None
    else:
        if tree is None:
            tree = ConstructTree(pos, m, softening, quadrupole=quadrupole)
            checkTreeQuadrupoles(tree, quadrupole)
            res = tree.fields(potential=key == "potential", accel=key == "accel", tidal=key == "tidal",
                              quadrupole=quadrupole, group_size=group_size, theta=theta, G=G, order="tree",
                              precision=precision, grouping=grouping, learned=learned,
                              error_ratio=error_ratio)[key]
        else:
            _check_tree(tree)
            checkTreeQuadrupoles(tree, quadrupole)
            # targets sorted by their own Morton order, not the tree's stored permutation (with
            # grouping="tree" or learned=True, grouped by their own octree)
            res = tree.fields(pos, softening, potential=key == "potential", accel=key == "accel",
                              tidal=key == "tidal", quadrupole=quadrupole, group_size=group_size, theta=theta, G=G,
                              order="morton", precision=precision, grouping=grouping, learned=learned,
                              error_ratio=error_ratio)[key]
    if return_tree:
        return res, tree
    return res


def _target_field(key, pos_target, pos_source, m_source, softening_target, softening_source, G, theta, tree,
                  return_tree, method, quadrupole, group_size, precision, grouping="blocks", learned=None,
                  error_ratio=None):
    valueTestMethod(method)
    if tree is None and (pos_source is None or m_source is None):
        raise ValueError("Must pass either pos_source & m_source or source tree.")
    pos_target = np.atleast_2d(_f64(pos_target))
    if softening_target is None:
        softening_target = zeros(len(pos_target))
    softening_target = np.atleast_1d(_f64(softening_target))
    if pos_source is not None:
        pos_source = np.atleast_2d(_f64(pos_source))
        m_source = np.atleast_1d(_f64(m_source))
        if softening_source is None:
            softening_source = zeros(len(pos_source))
        softening_source = np.atleast_1d(_f64(softening_source))
    if method == "adaptive":
        if pos_source is None or len(pos_target) * len(pos_source) > 10**6:
            method = "tree"
        else:
            method = "bruteforce"
    if method == "bruteforce":
        res = bruteforce(pos_target, softening_target, pos_source, m_source, softening_source, mutual=False, G=G,
                         precision="fp64", **{key: True})[key]
        if return_tree:
            tree = None
    else:
        if tree is None:
            tree = ConstructTree(pos_source, m_source, softening_source, quadrupole=quadrupole)
        _check_tree(tree)
        checkTreeQuadrupoles(tree, quadrupole)
        res = tree.fields(pos_target, softening_target, potential=key == "potential", accel=key == "accel",
                          tidal=key == "tidal", quadrupole=quadrupole, group_size=group_size, theta=theta, G=G,
                          order="morton", precision=precision, grouping=grouping, learned=learned,
                          error_ratio=error_ratio)[key]
    if return_tree:
        return res, tree
    return res


def Potential(pos, m, softening=None, G=1.0, theta=0.7, tree=None, return_tree=False, parallel=False,
              method="adaptive", quadrupole=False, group_size=8, device="cpu", *, precision="fp32",
              grouping="blocks", learned=None, error_ratio=None):
    """Gravitational potential of N particles at their own positions (frontend.py:145-293)."""
    return _self_field("potential", pos, m, softening, G, theta, tree, return_tree, method, quadrupole, group_size,
                       device, precision, 4000 if parallel else 1000, grouping, learned, error_ratio)


def Accel(pos, m, softening=None, G=1.0, theta=0.7, tree=None, return_tree=False, parallel=False,
          method="adaptive", quadrupole=False, group_size=8, device="cpu", *, precision="fp32", grouping="blocks",
          learned=None, error_ratio=None):
    """Gravitational acceleration of N particles at their own positions (frontend.py:421-560)."""
    return _self_field("accel", pos, m, softening, G, theta, tree, return_tree, method, quadrupole, group_size,
                       device, precision, 4000 if parallel else 1000, grouping, learned, error_ratio)


def TidalTensor(pos, m, softening=None, G=1.0, theta=0.7, tree=None, return_tree=False, parallel=False,
                method="adaptive", quadrupole=False, group_size=8, *, precision="fp32", grouping="blocks",
                learned=None, error_ratio=None):
    """Tidal tensor T_ij = dg_i/dx_j at the particle positions (frontend.py:688-789)."""
    return _self_field("tidal", pos, m, softening, G, theta, tree, return_tree, method, quadrupole, group_size,
                       None, precision, 4000 if parallel else 1000, grouping, learned, error_ratio)


def PotentialTarget(pos_target, pos_source, m_source, softening_target=None, softening_source=None, G=1.0,
                    theta=0.7, tree=None, return_tree=False, parallel=False, method="adaptive", quadrupole=False,
                    group_size=8, *, precision="fp32", grouping="blocks", learned=None,
                    error_ratio=None):
    """Potential at arbitrary target points from a set of sources (frontend.py:296-418)."""
    return _target_field("potential", pos_target, pos_source, m_source, softening_target, softening_source, G, theta,
                         tree, return_tree, method, quadrupole, group_size, precision, grouping, learned, error_ratio)


def AccelTarget(pos_target, pos_source, m_source, softening_target=None, softening_source=None, G=1.0, theta=0.7,
                tree=None, return_tree=False, parallel=False, method="adaptive", quadrupole=False, group_size=8, *,
                precision="fp32", grouping="blocks", learned=None,
                error_ratio=None):
    """Acceleration at arbitrary target points from a set of sources (frontend.py:563-685)."""
    return _target_field("accel", pos_target, pos_source, m_source, softening_target, softening_source, G, theta,
                         tree, return_tree, method, quadrupole, group_size, precision, grouping, learned, error_ratio)


def TidalTensorTarget(pos_target, pos_source, m_source, softening_target=None, softening_source=None, G=1.0,
                      theta=0.7, tree=None, return_tree=False, parallel=False, method="adaptive", quadrupole=False,
                      group_size=8, *, precision="fp32", grouping="blocks", learned=None,
                      error_ratio=None):
    """Tidal tensor at arbitrary target points from a set of sources (frontend.py:792-901)."""
    return _target_field("tidal", pos_target, pos_source, m_source, softening_target, softening_source, G, theta,
                         tree, return_tree, method, quadrupole, group_size, precision, grouping, learned, error_ratio)


class Field:
    """A reusable gravitational field: tree built once on the GPU, evaluated many times, any subset of
    potential/accel/tidal from a single traversal (frontend.py:904-1044)."""

    def __init__(self, pos, m, softening=None, G=1.0, theta=0.7, quadrupole=False, group_size=8, parallel=False, *,
                 precision="fp32", grouping="blocks", learned=None, error_ratio=None):
        pos = np.atleast_2d(_f64(pos))
        m = np.atleast_1d(_f64(m))
        if softening is None:
            softening = np.zeros_like(m)
        softening = np.atleast_1d(_f64(softening))
        self.G = G
        self.theta = theta
        self.quadrupole = quadrupole
        self.group_size = group_size
        self.parallel = parallel
        self.precision = precision
        self.grouping = grouping
        self.learned = learned
        self.error_ratio = error_ratio
        self.tree = ConstructTree(pos, m, softening, quadrupole=quadrupole)

    def __repr__(self):
        return (f"<pytreegrav.Field: {self.tree.NumParticles} particles, "
                f"{'quadrupole' if self.quadrupole else 'monopole'}, theta={self.theta}, "
                f"G={self.G}, group_size={self.group_size}, parallel={self.parallel}>")

    def evaluate(self, potential=False, accel=False, tidal=False, pos_target=None, softening_target=None, theta=None,
                 parallel=None, group_size=None, precision=None):
        if not (potential or accel or tidal):
            raise ValueError("request at least one of potential=True, accel=True, tidal=True")
        theta = self.theta if theta is None else theta
        group_size = self.group_size if group_size is None else group_size
        precision = self.precision if precision is None else precision
        kw = dict(potential=potential, accel=accel, tidal=tidal, quadrupole=self.quadrupole, group_size=group_size,
                  theta=theta, G=self.G, precision=precision)
        if pos_target is None:
            return self.tree.fields(order="tree", grouping=self.grouping, learned=self.learned,
                                    error_ratio=self.error_ratio, **kw)
        pos_target = np.atleast_2d(_f64(pos_target))
        if softening_target is None:
            softening_target = zeros(len(pos_target))
        softening_target = np.atleast_1d(_f64(softening_target))
        return self.tree.fields(pos_target, softening_target, order="morton", grouping=self.grouping,
                                learned=self.learned, error_ratio=self.error_ratio, **kw)

    def potential(self, pos_target=None, **kwargs):
        return self.evaluate(potential=True, pos_target=pos_target, **kwargs)["potential"]

    def accel(self, pos_target=None, **kwargs):
        return self.evaluate(accel=True, pos_target=pos_target, **kwargs)["accel"]

    def tidal(self, pos_target=None, **kwargs):
        return self.evaluate(tidal=True, pos_target=pos_target, **kwargs)["tidal"]


COLUMN_GROUP_MIN_TARGETS = 1000  # treewalk.py:16-19: from this many targets the binned walk is grouped


def ColumnDensity(pos, m, radii, rays=None, randomize_rays=False, healpix=False, tree=None, theta=0.5,
                  return_tree=False, parallel=False, group_size=16, device="cpu"):
    """Column density from each particle integrated to infinity, the particles being uniform spheres
    of mass m and radius radii (frontend.py:1321-1458): ray-traced along the given rays (int 6: the
    six axis rays; other ints: that many random directions; (N_rays, 3) array: normalised), or
    averaged over six bins on the sky with rays=None (opening angle theta). randomize_rays rotates
    the ray grid per particle by random_rotation(i) of its position i in Morton order. Returns
    (N, N_rays) or (N, 6) in the caller's order.

    The walks run on the GPU in FP64 in pytreegrav's order of operations (device and parallel are
    accepted; device keeps pytreegrav's checks), and the dispatch is pytreegrav's: the binned estimator
    walks per target below COLUMN_GROUP_MIN_TARGETS targets and by groups of group_size (at most 32
    here) from there on. The ray-traced walk does not depend on group_size (pytreegrav's grouped ray
    walk is bit-identical to its per-target one).
    """
    from .misc import random_rotation

    if np.any(np.asarray(radii) <= 0):
        warnings.warn("Some particle radii are <= 0; these particles are point-like and contribute no column "
                      "density. Supply a nonzero radius if their mass should be included.")
    pos = np.atleast_2d(_f64(pos))
    own = tree is None  # targets are the new tree's own particles: ordered and restored on the device
    if own:
        tree = ConstructTree(pos, _f64(m), _f64(radii))
        npos = len(pos)
    else:
        _check_tree(tree)
        idx = morton_order(pos)
        pos_sorted = np.ascontiguousarray(pos[idx])
        npos = len(pos_sorted)

    if type(rays) == int:
        if rays == 6:
            rays = np.vstack([np.eye(3), -np.eye(3)])
        else:
            rays = np.random.normal(size=(rays, 3))
    elif type(rays) == np.ndarray:
        if not len(rays.shape) == 2:
            raise Exception("rays array argument must be 2D.")
        elif rays.shape[1] != 3:
            raise Exception("rays array argument is not an array of 3D vectors.")
        rays = np.array(rays, dtype=np.float64)
    elif rays is not None:
        raise Exception("rays argument type is not supported")
    if healpix:
        try:
            import healpy as hp
        except ImportError as e:
            raise ImportError("healpix=... needs healpy: pip install healpy") from e
        nside = healpix
        rays = np.array(hp.pix2vec(nside, np.arange(hp.nside2npix(nside)))).T
    if rays is not None:
        rays /= np.sqrt((rays * rays).sum(1))[:, None]

    if device not in ("cpu", "cuda"):
        raise ValueError(f"device must be 'cpu' or 'cuda', got {device!r}")
    if device == "cuda" and (rays is None or randomize_rays):
        raise ValueError("device='cuda' supports only the ray-traced path: pass rays, and not randomize_rays")

    # the walks over the new tree's own particles return rows already in the caller's order
    walk = tree.column_density_self if own else (lambda *a: tree.column_density(pos_sorted, *a))
    if rays is None:  # pytreegrav groups the binned walk from COLUMN_GROUP_MIN_TARGETS targets on
        grouped = npos >= COLUMN_GROUP_MIN_TARGETS
        if grouped and not 1 <= group_size <= 32:
            raise ValueError("group_size must be between 1 and 32 for the grouped binned walk")
        columns = walk(None, theta, group_size if grouped else 0)
    elif randomize_rays:
        per = np.empty((npos,) + rays.shape)
        for i in range(npos):
            per[i] = rays @ random_rotation(i)
        columns = walk(per)
    else:
        columns = walk(rays)
    if device == "cuda":  # pytreegrav's device path returns float32
        columns = columns.astype(np.float32)
    if np.any(np.isnan(columns)):
        print("WARNING some column densities are NaN!")
    if own:
        unsorted = columns
    else:
        unsorted = np.empty_like(columns)
        unsorted[idx] = columns
    if return_tree:
        return unsorted, tree
    return unsorted


def _default_rbins(pos):
    """frontend.py:1091-1093: log-spaced edges from the 11th-nearest to the farthest distance from the
    median position, N^(1/3) of them. The two order statistics come from a partition and a maximum
    (the same values as pytreegrav's full sort, in linear time)."""
    # per contiguous column: numpy's median and the same sum of squares as np.sum(d ** 2, axis=1)
    cols = [np.ascontiguousarray(pos[:, k]) for k in range(pos.shape[1])]
    d = [c - np.median(c) for c in cols]
    r = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) if len(d) == 3 else \
        np.sqrt(np.sum((pos - np.median(pos, axis=0)) ** 2, axis=1))
    if len(r) <= 10:
        r = np.sort(r)  # too few points: pytreegrav's own failure (an IndexError) below
        return 10 ** np.linspace(np.log10(r[10]), np.log10(r[-1]), int(len(r) ** (1.0 / 3)))
    return 10 ** np.linspace(np.log10(np.partition(r, 10)[10]), np.log10(r.max()), int(len(r) ** (1.0 / 3)))


def _corr(kind, pos, m, v, rbins, max_bin_size_ratio, theta, tree, boxsize, weighted_binning, seed):
    """The frontends' common path (frontend.py:1090-1130, 1176-1224, 1270-1318): targets are the
    tree's own particles in walk order when the tree is built here (no host gather: the library
    reads them, their velocities and masses from the tree), else pos in its own Morton order."""
    pos = np.atleast_2d(_f64(pos))
    if rbins is None:
        rbins = _default_rbins(pos)
    rbins = np.ascontiguousarray(_f64(rbins))
    if tree is None:
        tree = ConstructTree(pos, _f64(m), zeros(len(pos)), vel=v)
        bs, ws = tree.correlation(kind, None, rbins, max_bin_size_ratio=max_bin_size_ratio, theta=theta,
                                  boxsize=boxsize, weighted_binning=weighted_binning, seed=seed)
    else:
        _check_tree(tree)
        idx = morton_order(pos)
        vs = ms = None
        if v is not None:
            vs = np.take(np.atleast_2d(_f64(v)), idx, axis=0)
            ms = np.take(np.atleast_1d(_f64(m)), idx, axis=0)
        bs, ws = tree.correlation(kind, np.take(pos, idx, axis=0), rbins, vel=vs, weight=ms,
                                  max_bin_size_ratio=max_bin_size_ratio, theta=theta, boxsize=boxsize,
                                  weighted_binning=weighted_binning, seed=seed)
    return rbins, bs, ws, tree


def DensityCorrFunc(pos, m, rbins=None, max_bin_size_ratio=100, theta=1.0, tree=None, return_tree=False,
                    parallel=False, boxsize=0, weighted_binning=False, *, seed=None):
    """Mean mass in logarithmic radial bins around each point, averaged over the points
    (frontend.py:1047-1130; treewalk.py:378-510): returns (rbins, mbins[, tree]).

    rbins None: N^(1/3) log-spaced edges from the points' spread about their median. A node is
    binned whole once it passes the opening test at theta and is smaller than max_bin_size_ratio
    bin widths: spread over the bins it overlaps (weighted_binning) or at a distance jittered by its
    size (keyed by seed). Periodic when boxsize > 0. tree: any tree (not necessarily of pos).
    The walks run on the GPU in FP64 (one thread per target).
    """
    rbins, bs, _, tree = _corr("density", pos, m, None, rbins, max_bin_size_ratio, theta, tree, boxsize,
                               weighted_binning, seed)
    mbins = bs / len(np.atleast_2d(pos))
    return (rbins, mbins, tree) if return_tree else (rbins, mbins)


def VelocityCorrFunc(pos, m, v, rbins=None, max_bin_size_ratio=100, theta=1.0, tree=None, return_tree=False,
                     parallel=False, boxsize=0, weighted_binning=False, *, seed=None):
    """Mass-weighted mean of v . v' in logarithmic radial bins, averaged over the points
    (frontend.py:1133-1224; treewalk.py:515-663): returns (rbins, corr[, tree]). A given tree must
    carry velocities (ConstructTree(..., vel=...)); v may be any vector field. Arguments as
    DensityCorrFunc."""
    rbins, bs, ws, tree = _corr("velocity", pos, m, v, rbins, max_bin_size_ratio, theta, tree, boxsize,
                                weighted_binning, seed)
    with np.errstate(invalid="ignore", divide="ignore"):
        corr = bs / ws
    return (rbins, corr, tree) if return_tree else (rbins, corr)


def VelocityStructFunc(pos, m, v, rbins=None, max_bin_size_ratio=100, theta=1.0, tree=None, return_tree=False,
                       parallel=False, boxsize=0, weighted_binning=False, *, seed=None):
    """Mass-weighted mean of |v - v'|^2 in logarithmic radial bins, averaged over the points, a
    node's own velocity dispersion included (frontend.py:1227-1318; treewalk.py:668-818): returns
    (rbins, Sv[, tree]). Arguments as VelocityCorrFunc."""
    rbins, bs, ws, tree = _corr("structure", pos, m, v, rbins, max_bin_size_ratio, theta, tree, boxsize,
                                weighted_binning, seed)
    with np.errstate(invalid="ignore", divide="ignore"):
        Sv = bs / ws
    return (rbins, Sv, tree) if return_tree else (rbins, Sv)
