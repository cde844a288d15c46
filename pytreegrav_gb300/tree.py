"""Device-resident octree with pytreegrav's Octree interface (src/pytreegrav/octree.py:8-28, 664-723).

The tree lives on the GPU as the arrays pytreegrav defines -- particles at [0, NumParticles) in
Morton order, nodes after them in pytreegrav's own numbering -- plus a walk arena derived from them.
The attribute arrays (Coordinates, Masses, ...) are copied to the host on first access, padded to
NumNodes rows exactly as pytreegrav leaves its spare capacity (zeros, and -1 links).
"""

import ctypes

import numpy as np

from . import _lib

FIELD_KEYS = ("potential", "accel", "tidal")


def _as_f64(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        a = a.reshape(shape)
    return a


_MODELS = {}  # learned opening-test models by the `learned` argument that named them


class Octree:
    """An octree built on the GPU by ConstructTree.

    Attributes mirror pytreegrav's Octree jitclass: NumParticles, NumNodes, HasQuads,
    HasCoincidentPoints, Coordinates, Masses, Sizes, Deltas, Softenings, Quadrupoles,
    FirstSubnode, NextBranch, TreewalkIndices; and, for a tree built with velocities (the
    DynamicOctree's role), Velocities and VelocityDisp.
    """

    HasVelocities = False

    def __init__(self, pos, m=None, softening=None, quadrupole=False, compute_moments=True):
        L = _lib.load()
        pos = _as_f64(pos, (-1, 3))
        n = len(pos)
        m = None if m is None else _as_f64(m, (n,))
        softening = None if softening is None else _as_f64(softening, (n,))
        handle = ctypes.c_void_p()
        rc = L.tg_tree_build(_lib.ptr(pos), _lib.ptr(m), _lib.ptr(softening), n, int(bool(quadrupole)),
                             int(bool(compute_moments)), _lib.TG_MEM_HOST, None, ctypes.byref(handle))
        _lib.check(rc, "ConstructTree")
        self._h = handle
        self._host = None
        info = _lib.TreeInfo()
        _lib.check(L.tg_tree_info_get(self._h, ctypes.byref(info)))
        self.NumParticles = int(info.npart)
        self.NumNodes = int(info.num_nodes)
        self.node_hi = int(info.node_hi)
        self.HasQuads = bool(quadrupole)
        self.HasCoincidentPoints = bool(info.has_coincident)

    @classmethod
    def _from_handle(cls, handle, quadrupole):
        self = cls.__new__(cls)
        L = _lib.load()
        self._h = handle
        self._host = None
        info = _lib.TreeInfo()
        _lib.check(L.tg_tree_info_get(self._h, ctypes.byref(info)))
        self.NumParticles = int(info.npart)
        self.NumNodes = int(info.num_nodes)
        self.node_hi = int(info.node_hi)
        self.HasQuads = bool(quadrupole)
        self.HasCoincidentPoints = bool(info.has_coincident)
        return self

    @classmethod
    def batched(cls, pos, m, softening, offsets, quadrupole=False):
        """Independent systems stored back to back (system s owns rows offsets[s]:offsets[s+1]) in
        one tree arena from one segmented build (no counterpart in pytreegrav)."""
        L = _lib.load()
        pos = _as_f64(pos, (-1, 3))
        n = len(pos)
        m = _as_f64(m, (n,))
        softening = np.zeros(n) if softening is None else _as_f64(softening, (n,))
        offsets = np.ascontiguousarray(offsets, np.int64)
        handle = ctypes.c_void_p()
        rc = L.tg_tree_build_batched(_lib.ptr(pos), _lib.ptr(m), _lib.ptr(softening), _lib.ptr(offsets),
                                     len(offsets) - 1, int(bool(quadrupole)), _lib.TG_MEM_HOST, None,
                                     ctypes.byref(handle))
        _lib.check(rc, "batched build")
        return cls._from_handle(handle, quadrupole)

    def set_walk_config(self, warps_per_block=4, first_stack=1024):
        """Launch shape of this tree's walks (see tg_tree_set_walk_config); results do not depend on it."""
        _lib.check(_lib.load().tg_tree_set_walk_config(self._h, int(warps_per_block), int(first_stack)),
                   "walk config")

    def walk_graph(self, out, potential=False, accel=False, tidal=False, quadrupole=False, group_size=32,
                   theta=0.7, G=1.0, grouping="tree"):
        """The walk of this tree's own particles captured in a CUDA graph (tg_walk_graph_*), writing
        to `out`, a device array of NumParticles x W float64 (an integer address or an object with
        data_ptr()) that must outlive the graph."""
        return WalkGraph(self, out, potential, accel, tidal, quadrupole, group_size, theta, G, grouping)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().tg_tree_free(h)
            except Exception:
                pass
            self._h = None

    # -- host copies of the Octree arrays ------------------------------------------------------
    def _arrays(self):
        if self._host is None:
            nn, n = self.NumNodes, self.NumParticles
            a = {
                "Coordinates": np.empty((nn, 3)),
                "Masses": np.empty(nn),
                "Sizes": np.empty(nn),
                "Deltas": np.empty(nn),
                "Softenings": np.empty(nn),
                "Quadrupoles": np.empty((nn, 3, 3)) if self.HasQuads else None,
                "FirstSubnode": np.empty(nn, np.int64),
                "NextBranch": np.empty(nn, np.int64),
                "TreewalkIndices": np.empty(n, np.int64),
            }
            p = _lib.ptr
            rc = _lib.load().tg_tree_copy_out(self._h, p(a["Coordinates"]), p(a["Masses"]), p(a["Sizes"]),
                                              p(a["Deltas"]), p(a["Softenings"]), p(a["Quadrupoles"]),
                                              p(a["FirstSubnode"]), p(a["NextBranch"]), p(a["TreewalkIndices"]),
                                              None)
            _lib.check(rc, "copy_out")
            self._host = a
        return self._host

    def __getattr__(self, name):
        if name in ("Coordinates", "Masses", "Sizes", "Deltas", "Softenings", "Quadrupoles", "FirstSubnode",
                    "NextBranch", "TreewalkIndices"):
            return self._arrays()[name]
        raise AttributeError(name)

    # -- evaluation ------------------------------------------------------------------------------
    def fields(self, pos=None, soft=None, potential=False, accel=False, tidal=False, quadrupole=False,
               group_size=8, theta=0.7, G=1.0, order="tree", precision="fp32", theta_per_group=None,
               grouping="blocks", learned=None, error_ratio=None):
        """Any subset of {potential, accel, tidal} from one traversal (FieldsTarget_grouped).

        order="tree": the tree's own particles are the targets (pos/soft ignored); "morton": targets
        are Morton-sorted by their own bounding cube before grouping; "given": grouped as passed.
        grouping="blocks": group_size consecutive targets per group (pytreegrav's grouping);
        "tree": groups taken from the tree (order="tree"), or, for order="morton", from an octree
        of the targets themselves (see TargetSet).
        learned (extension): True for the packaged opening-angle model, a path or a
        theta.ThetaModel -- the acceptance test of each group then comes from the network
        (tree grouping of 32, FP32; order="tree", or order="morton" through a TargetSet);
        error_ratio asks for that RMS force error
        relative to the plain walk at theta = 0.7 (default: the model's calibrated lambda), and
        `theta` is the fallback angle.
        Results come back in the caller's order (the tree's input order for order="tree").
        """
        if order == "morton" and ((learned is not None and learned is not False) or grouping == "tree"):
            # external targets grouped by their own octree (tg_targets_*)
            ts = TargetSet(self, pos, soft, group_size=32 if learned not in (None, False) else group_size)
            try:
                if learned is not None and learned is not False:
                    return ts.fields_learned(potential, accel, tidal, quadrupole, theta, G, precision, learned,
                                             error_ratio)
                return ts.fields(potential, accel, tidal, quadrupole, theta, G, precision)
            finally:
                ts.close()
        if learned is not None and learned is not False:
            return self._fields_learned(potential, accel, tidal, quadrupole, theta, G, order, precision, learned,
                                        error_ratio)
        fields = (_lib.TG_FIELD_POTENTIAL * bool(potential) + _lib.TG_FIELD_ACCEL * bool(accel)
                  + _lib.TG_FIELD_TIDAL * bool(tidal))
        if fields == 0:
            raise ValueError("request at least one of potential=True, accel=True, tidal=True")
        if quadrupole and not self.HasQuads:
            _lib.check(_lib.TG_ERR_NO_QUADRUPOLES)
        W = int(bool(potential)) + 3 * int(bool(accel)) + 9 * int(bool(tidal))
        ord_code = {"tree": _lib.TG_ORDER_TREE, "morton": _lib.TG_ORDER_MORTON, "given": _lib.TG_ORDER_GIVEN}[order]
        prec = {"fp32": _lib.TG_FP32, "fp64": _lib.TG_FP64}[precision]
        if ord_code == _lib.TG_ORDER_TREE:
            n = self.NumParticles
            pos_p = soft_p = None
        else:
            pos = _as_f64(pos, (-1, 3))
            n = len(pos)
            soft = np.zeros(n) if soft is None else _as_f64(soft, (n,))
            pos_p, soft_p = _lib.ptr(pos), _lib.ptr(soft)
        out = np.empty((n, W))
        if n == 0:
            return _split(out, potential, accel, tidal)
        tpg = None
        if theta_per_group is not None:
            tpg = ctypes.c_void_p(int(theta_per_group))  # a device pointer (float32, one per group)
        grp = {"blocks": _lib.TG_GROUP_BLOCKS, "tree": _lib.TG_GROUP_TREE}[grouping]
        rc = _lib.load().tg_tree_fields(self._h, pos_p, soft_p, n, fields, int(bool(quadrupole)), float(theta),
                                        float(G), int(group_size), grp, ord_code, prec, tpg, _lib.TG_MEM_HOST,
                                        _lib.ptr(out), None)
        _lib.check(rc, "tree walk")
        return _split(out, potential, accel, tidal)

    def _fields_learned(self, potential, accel, tidal, quadrupole, theta, G, order, precision, learned, error_ratio):
        from . import theta as th

        if order != "tree":
            raise ValueError("the learned opening test evaluates the tree's own particles (order='tree')")
        if precision != "fp32":
            raise ValueError("the learned opening test runs the FP32 walk")
        fields = (_lib.TG_FIELD_POTENTIAL * bool(potential) + _lib.TG_FIELD_ACCEL * bool(accel)
                  + _lib.TG_FIELD_TIDAL * bool(tidal))
        if fields == 0:
            raise ValueError("request at least one of potential=True, accel=True, tidal=True")
        if quadrupole and not self.HasQuads:
            _lib.check(_lib.TG_ERR_NO_QUADRUPOLES)
        model, l10 = _model_and_lambda(learned, error_ratio, quadrupole)
        W = int(bool(potential)) + 3 * int(bool(accel)) + 9 * int(bool(tidal))
        out = np.empty((self.NumParticles, W))
        rc = _lib.load().tg_tree_fields_learned(self._h, fields, int(bool(quadrupole)), float(G), th.GROUP_SIZE,
                                                model.handle(), float(l10), float(theta), _lib.TG_MEM_HOST,
                                                _lib.ptr(out), None)
        _lib.check(rc, "learned tree walk")
        return _split(out, potential, accel, tidal)

    def column_density(self, pos, rays=None, theta=0.5, group_size=0):
        """Column density of this tree's particles (uniform spheres, radius = softening) from each
        target to infinity (tg_tree_column_density). rays: (nrays, 3) unit vectors shared by all
        targets, or (n, nrays, 3) per target, -> (n, nrays) from the ray-traced walk; None -> (n, 6)
        from the angle-binned walk at opening angle theta, per target (group_size 0) or grouped by
        group_size consecutive targets. Targets are taken in the order given."""
        pos = _as_f64(pos, (-1, 3))
        n = len(pos)
        if rays is None:
            out = np.empty((n, 6))
            rc = _lib.load().tg_tree_column_density(self._h, _lib.ptr(pos), n, None, 0, 0, 1, float(theta),
                                                    int(group_size), _lib.TG_MEM_HOST, _lib.ptr(out), None)
        else:
            rays = np.ascontiguousarray(rays, np.float64)
            per_target = rays.ndim == 3
            nrays = rays.shape[-2]
            if rays.shape[-1] != 3 or (per_target and rays.shape[0] != n):
                raise ValueError("rays must be (nrays, 3), or (n, nrays, 3) for per-target rays")
            out = np.empty((n, nrays))
            rc = _lib.load().tg_tree_column_density(self._h, _lib.ptr(pos), n, _lib.ptr(rays), nrays,
                                                    3 * nrays if per_target else 0, 0, 0.0, 0, _lib.TG_MEM_HOST,
                                                    _lib.ptr(out), None)
        _lib.check(rc, "column density")
        return out

    def column_density_self(self, rays=None, theta=0.5, group_size=0):
        """column_density with this tree's own particles as the targets, taken in walk (Morton)
        order on the device; per-target rays (NumParticles, nrays, 3) are in that order too. The
        rows come back in the caller's original particle order (TreewalkIndices undone on the
        device), so no host gather or scatter is needed."""
        n = self.NumParticles
        L = _lib.load()
        if rays is None:
            out = np.empty((n, 6))
            rc = L.tg_tree_column_density(self._h, None, n, None, 0, 0, 1, float(theta), int(group_size),
                                          _lib.TG_MEM_HOST, _lib.ptr(out), None)
        else:
            rays = np.ascontiguousarray(rays, np.float64)
            per_target = rays.ndim == 3
            nrays = rays.shape[-2]
            if rays.shape[-1] != 3 or (per_target and rays.shape[0] != n):
                raise ValueError("rays must be (nrays, 3), or (n, nrays, 3) for per-target rays")
            out = np.empty((n, nrays))
            rc = L.tg_tree_column_density(self._h, None, n, _lib.ptr(rays), nrays, 3 * nrays if per_target else 0,
                                          0, 0.0, 0, _lib.TG_MEM_HOST, _lib.ptr(out), None)
        _lib.check(rc, "column density")
        return out

    # -- velocities and two-point functions -----------------------------------------------------
    def set_velocities(self, vel):
        """Attach particle velocities (n, 3), caller's order, and roll up every node's mass-weighted
        mean velocity and velocity dispersion as pytreegrav's DynamicOctree does
        (dynamic_tree.py:246-310; tg_tree_set_velocities)."""
        vel = _as_f64(vel, (-1, 3))
        if len(vel) != self.NumParticles:
            raise ValueError(f"vel has {len(vel)} rows for a tree of {self.NumParticles} particles")
        _lib.check(_lib.load().tg_tree_set_velocities(self._h, _lib.ptr(vel), _lib.TG_MEM_HOST, None),
                   "tree velocities")
        self._vel = None
        self.HasVelocities = True

    def _velocities(self):
        if not getattr(self, "HasVelocities", False):
            raise AttributeError("this tree has no velocities (ConstructTree(..., vel=v))")
        if getattr(self, "_vel", None) is None:
            v, d = np.empty((self.NumNodes, 3)), np.empty(self.NumNodes)
            _lib.check(_lib.load().tg_tree_copy_velocities(self._h, _lib.ptr(v), _lib.ptr(d), None),
                       "copy velocities")
            self._vel = (v, d)
        return self._vel

    @property
    def Velocities(self):
        """(NumNodes, 3): particle velocities (tree order) and nodes' mass-weighted mean velocities."""
        return self._velocities()[0]

    @property
    def VelocityDisp(self):
        """(NumNodes,): nodes' mass-weighted velocity dispersions (particles 0)."""
        return self._velocities()[1]

    def correlation(self, kind, pos, rbins, vel=None, weight=None, max_bin_size_ratio=100, theta=1.0, boxsize=0,
                    weighted_binning=False, seed=None):
        """Sums of the density / velocity-correlation / structure-function walks of the targets pos
        (taken in the order given) over this tree (tg_tree_correlation): (binsums, wtsums), nbins each.
        pos=None: the tree's own particles in tree order, weighted by their masses, with their own
        velocities (vel and weight ignored). seed: the jitter stream's key (None: drawn from numpy's
        global generator)."""
        k = _lib.TG_CORR_KINDS[kind]
        if k and not self.HasVelocities:
            raise ValueError(f"the {kind} function needs a tree with velocities: ConstructTree(..., vel=v)")
        rbins = _as_f64(rbins)
        nb = len(rbins) - 1
        if nb < 1 or nb > _lib.TG_CORR_MAX_BINS:
            raise ValueError(f"rbins must hold 2 to {_lib.TG_CORR_MAX_BINS + 1} edges")
        if not (rbins[0] > 0 and np.all(np.diff(rbins) > 0)):
            raise ValueError("rbins must be positive and increasing (logarithmically spaced)")
        vp = wp = pp = None
        n = self.NumParticles
        if pos is not None:
            pos = _as_f64(pos, (-1, 3))
            n = len(pos)
            pp = _lib.ptr(pos)
            if k:
                vel = _as_f64(vel, (n, 3))
                weight = _as_f64(weight, (n,))
                vp, wp = _lib.ptr(vel), _lib.ptr(weight)
        if seed is None:
            seed = int(np.random.randint(0, 2**63 - 1, dtype=np.int64))
        bs, ws = np.zeros(nb), np.zeros(nb)
        rc = _lib.load().tg_tree_correlation(self._h, k, pp, vp, wp, n, _lib.ptr(rbins), nb,
                                             float(max_bin_size_ratio), float(theta), float(boxsize),
                                             int(bool(weighted_binning)), int(seed) & (2**64 - 1),
                                             _lib.TG_MEM_HOST, _lib.ptr(bs), _lib.ptr(ws), None)
        _lib.check(rc, "correlation walk")
        return bs, ws

    def last_walk_stats(self):
        """(interactions, node tests, deepest stack, groups) of the last walk on this tree."""
        v = [ctypes.c_int64() for _ in range(4)]
        _lib.check(_lib.load().tg_tree_last_walk_stats(self._h, *[ctypes.byref(x) for x in v]))
        return tuple(int(x.value) for x in v)


def _model_and_lambda(learned, error_ratio, quadrupole, targets=False):
    """The ThetaModel named by `learned` (True: the packaged model; a path; or a model) and the log10
    lambda that gives `error_ratio` (None: the model's calibrated default) for the tree's own
    particles or, with targets=True, for external targets."""
    from . import theta as th

    if isinstance(learned, th.ThetaModel):
        model = learned
    else:
        model = _MODELS.get(learned)
        if model is None:  # loaded and uploaded once per process, shared by every tree
            model = th.ThetaModel.load(None if learned is True else learned)
            _MODELS[learned] = model
    l10 = (th.default_lambda(model, quadrupole, targets) if error_ratio is None
           else th.lambda_for_ratio(model, float(error_ratio), quadrupole, targets))
    if l10 is None:
        l10 = th.default_lambda(model, quadrupole, targets)
    return model, l10


class TargetSet:
    """External target points prepared once for walks of one source tree (tg_targets_*; no
    counterpart in pytreegrav, which groups the Morton-sorted targets in consecutive blocks of
    group_size, grouped_treewalk.py:269-275). The targets get an octree of their own and are grouped
    by it: subtrees and runs of siblings of at most group_size targets, so that no group straddles a
    jump of the Morton curve. Results come back in the caller's order."""

    def __init__(self, tree, pos, soft=None, group_size=32):
        self.tree = tree  # the source tree must outlive the set
        pos = _as_f64(pos, (-1, 3))
        n = len(pos)
        soft = np.zeros(n) if soft is None else _as_f64(soft, (n,))
        self.n = n
        self.group_size = int(group_size)
        self._h = ctypes.c_void_p()
        if n:
            _lib.check(_lib.load().tg_targets_create(tree._h, _lib.ptr(pos), _lib.ptr(soft), n, self.group_size,
                                                     _lib.TG_MEM_HOST, None, ctypes.byref(self._h)), "target set")

    @property
    def handle(self):
        return self._h

    def ngroups(self):
        ng = ctypes.c_int64()
        if self._h.value:
            _lib.check(_lib.load().tg_targets_info(self._h, None, ctypes.byref(ng)), "target set")
        return int(ng.value)

    def groups(self):
        """(first, count, source node) per group (int32) and each walk-order target's caller index."""
        ng = self.ngroups()
        first, count, node = (np.empty(ng, np.int32) for _ in range(3))
        widx = np.empty(self.n, np.int64)
        if self.n:
            _lib.check(_lib.load().tg_targets_groups_copy(self._h, _lib.ptr(first), _lib.ptr(count), _lib.ptr(node),
                                                          _lib.ptr(widx), _lib.TG_MEM_HOST, None), "target groups")
        return first, count, node, widx

    def fields(self, potential=False, accel=False, tidal=False, quadrupole=False, theta=0.7, G=1.0, precision="fp32"):
        fields = (_lib.TG_FIELD_POTENTIAL * bool(potential) + _lib.TG_FIELD_ACCEL * bool(accel)
                  + _lib.TG_FIELD_TIDAL * bool(tidal))
        if fields == 0:
            raise ValueError("request at least one of potential=True, accel=True, tidal=True")
        if quadrupole and not self.tree.HasQuads:
            _lib.check(_lib.TG_ERR_NO_QUADRUPOLES)
        W = int(bool(potential)) + 3 * int(bool(accel)) + 9 * int(bool(tidal))
        out = np.empty((self.n, W))
        if self.n:
            prec = {"fp32": _lib.TG_FP32, "fp64": _lib.TG_FP64}[precision]
            _lib.check(_lib.load().tg_targets_fields(self._h, fields, int(bool(quadrupole)), float(theta), float(G),
                                                     prec, None, _lib.TG_MEM_HOST, _lib.ptr(out), None),
                       "target walk")
        return _split(out, potential, accel, tidal)

    def fields_learned(self, potential=False, accel=False, tidal=False, quadrupole=False, theta=0.7, G=1.0,
                       precision="fp32", learned=True, error_ratio=None):
        """The walk with each group's acceptance test from the learned model (see Octree.fields);
        theta is the fallback angle."""
        if precision != "fp32":
            raise ValueError("the learned opening test runs the FP32 walk")
        fields = (_lib.TG_FIELD_POTENTIAL * bool(potential) + _lib.TG_FIELD_ACCEL * bool(accel)
                  + _lib.TG_FIELD_TIDAL * bool(tidal))
        if fields == 0:
            raise ValueError("request at least one of potential=True, accel=True, tidal=True")
        if quadrupole and not self.tree.HasQuads:
            _lib.check(_lib.TG_ERR_NO_QUADRUPOLES)
        model, l10 = _model_and_lambda(learned, error_ratio, quadrupole, targets=True)
        W = int(bool(potential)) + 3 * int(bool(accel)) + 9 * int(bool(tidal))
        out = np.empty((self.n, W))
        if self.n:
            _lib.check(_lib.load().tg_targets_fields_learned(self._h, fields, int(bool(quadrupole)), float(G),
                                                             model.handle(), float(l10), float(theta),
                                                             _lib.TG_MEM_HOST, _lib.ptr(out), None),
                       "learned target walk")
        return _split(out, potential, accel, tidal)

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().tg_targets_free(h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WalkGraph:
    """A captured walk (see Octree.walk_graph): launch() replays it on a stream, status() waits and
    raises if the last replay failed."""

    def __init__(self, tree, out, potential, accel, tidal, quadrupole, group_size, theta, G, grouping):
        fields = (_lib.TG_FIELD_POTENTIAL * bool(potential) + _lib.TG_FIELD_ACCEL * bool(accel)
                  + _lib.TG_FIELD_TIDAL * bool(tidal))
        if fields == 0:
            raise ValueError("request at least one of potential=True, accel=True, tidal=True")
        self.tree = tree  # the graph reads the tree's arrays
        self.out = out
        addr = out.data_ptr() if hasattr(out, "data_ptr") else int(out)
        grp = {"blocks": _lib.TG_GROUP_BLOCKS, "tree": _lib.TG_GROUP_TREE}[grouping]
        self._g = ctypes.c_void_p()
        _lib.check(_lib.load().tg_walk_graph_create(tree._h, fields, int(bool(quadrupole)), float(theta), float(G),
                                                    int(group_size), grp, ctypes.c_void_p(addr),
                                                    ctypes.byref(self._g)), "walk graph")

    def launch(self, stream=None):
        _lib.check(_lib.load().tg_walk_graph_launch(self._g, stream), "walk graph launch")

    def status(self, stream=None):
        _lib.check(_lib.load().tg_walk_graph_status(self._g, stream), "walk graph")

    def close(self):
        g = getattr(self, "_g", None)
        if g is not None and g.value:
            _lib.load().tg_walk_graph_free(g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _split(out, potential, accel, tidal):
    res, o = {}, 0
    if potential:
        res["potential"] = out[:, 0].copy()
        o = 1
    if accel:
        res["accel"] = np.ascontiguousarray(out[:, o:o + 3])
        o += 3
    if tidal:
        res["tidal"] = np.ascontiguousarray(out[:, o:o + 9]).reshape(-1, 3, 3)
    return res


def morton_order(pos):
    """Stable permutation sorting points by Morton key in their own bounding cube (_morton_order)."""
    pos = _as_f64(pos, (-1, 3))
    perm = np.empty(len(pos), np.int64)
    if len(pos):
        _lib.check(_lib.load().tg_morton_order(_lib.ptr(pos), len(pos), _lib.TG_MEM_HOST, _lib.ptr(perm), None),
                   "morton_order")
    return perm


def bruteforce(pos_t, h_t, pos_s, m_s, h_s, potential=False, accel=False, tidal=False, mutual=False, G=1.0,
               precision="fp64"):
    """Direct summation on the GPU. mutual=True: targets are the sources, self excluded by index."""
    fields = 1 * bool(potential) + 2 * bool(accel) + 4 * bool(tidal)
    if fields == 0:
        raise ValueError("request at least one field")
    pos_s = _as_f64(pos_s, (-1, 3))
    ns = len(pos_s)
    m_s = _as_f64(m_s, (ns,))
    h_s = np.zeros(ns) if h_s is None else _as_f64(h_s, (ns,))
    if mutual:
        pos_t, h_t = pos_s, h_s
    else:
        pos_t = _as_f64(pos_t, (-1, 3))
        h_t = np.zeros(len(pos_t)) if h_t is None else _as_f64(h_t, (len(pos_t),))
    nt = len(pos_t)
    W = int(bool(potential)) + 3 * int(bool(accel)) + 9 * int(bool(tidal))
    out = np.empty((nt, W))
    if nt:
        prec = {"fp32": _lib.TG_FP32, "fp64": _lib.TG_FP64}[precision]
        rc = _lib.load().tg_bruteforce(_lib.ptr(pos_t), _lib.ptr(h_t), nt, _lib.ptr(pos_s), _lib.ptr(m_s),
                                       _lib.ptr(h_s), ns, fields, int(bool(mutual)), float(G), prec,
                                       _lib.TG_MEM_HOST, _lib.ptr(out), None)
        _lib.check(rc, "bruteforce")
    return _split(out, potential, accel, tidal)
