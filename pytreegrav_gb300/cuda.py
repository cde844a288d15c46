"""Device-resident gravity contexts under pytreegrav.cuda's names (cuda.py:546-611 for the tree
contexts, cuda.py:737-796 for the brute-force ones).

A context puts the tree, or the source set, on the GPU once; each call uploads one set of targets,
evaluates on the GPU and returns the result. Call signatures, defaults, float32 results and the
missing-device error follow pytreegrav.cuda. The work runs on this package's kernels. The tree
contexts use the octree walk, and the brute-force contexts the FP32 direct sum. There is no CPU path
here: without the library or a GPU the constructors raise.

As in pytreegrav.cuda, positions and softenings are narrowed to float32 on the way in, both for the
sources (the packed rows there) and for the targets (every call). A target that is one of the
sources therefore lands exactly on it, and the r == 0 test drops the self term.
"""

import ctypes

import numpy as np

from . import _lib
from .tree import Octree

THREADS_X = 32  # accepted for signature compatibility (cuda.py:38); the launch shape is the library's
GRAV_ROW = 8    # row width of pack_tree_gravity (cuda.py:305)

_NO_DEVICE = ("no CUDA device available. pytreegrav_gb300.cuda needs the compiled library "
              "(python -m pytreegrav_gb300.build) and a visible NVIDIA GPU.")


def is_available():
    """True if the library loads and a CUDA device is visible (cuda.py:70-80)."""
    try:
        L = _lib.load()
    except Exception:
        return False
    n = ctypes.c_int(0)
    try:
        return L.tg_device_count(ctypes.byref(n)) == _lib.TG_OK and n.value > 0
    except Exception:
        return False


def _require_device():
    if not is_available():
        raise RuntimeError(_NO_DEVICE)


def _f32(a, shape):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(shape))


def _soft32(softening, n):
    if softening is None:
        return np.zeros(n, dtype=np.float32)
    return np.ascontiguousarray(np.broadcast_to(np.asarray(softening, dtype=np.float32), (n,)))


def pack_tree_gravity(tree, dtype=np.float32):
    """The packed gravity rows of pytreegrav.cuda (cuda.py:299-357): (nodes (NumNodes, 8) `dtype`
    holding centre of mass, mass, softening, size, delta and a pad; links (NumNodes, 2) int32 holding
    NextBranch and FirstSubnode). A data-format helper; the contexts below do not need it."""
    n = int(tree.NumNodes)
    rows = np.zeros((n, GRAV_ROW), dtype=dtype)
    with np.errstate(over="ignore"):
        rows[:, 0:3] = np.asarray(tree.Coordinates[:n], dtype=np.float64)
        rows[:, 3] = np.asarray(tree.Masses[:n], dtype=np.float64)
        rows[:, 4] = np.asarray(tree.Softenings[:n], dtype=np.float64)
        rows[:, 5] = np.asarray(tree.Sizes[:n], dtype=np.float64)
        rows[:, 6] = np.asarray(tree.Deltas[:n], dtype=np.float64)
    links = np.empty((n, 2), dtype=np.int32)
    links[:, 0] = np.asarray(tree.NextBranch[:n])
    links[:, 1] = np.asarray(tree.FirstSubnode[:n])
    bad = ~np.isfinite(rows[:, :7])
    if bad.any():
        i, slot = np.argwhere(bad)[0]
        raise ValueError(f"packing overflowed {np.dtype(dtype).name} at {int(bad.sum())} entries "
                         f"(first: element {i}, slot {slot}).")
    return rows, links


class _CudaGravity:
    """Shared base of the tree contexts: the tree goes to the GPU once, every call walks it for a new
    set of targets (cuda.py:546-589). Monopole, float32 results."""

    _WIDTH = 1
    _KEY = "potential"

    def __init__(self, tree, threads_x=THREADS_X):
        _require_device()
        n = int(tree.NumParticles)
        pos = np.asarray(tree.Coordinates[:n], dtype=np.float64)
        pos32 = pos.astype(np.float32).astype(np.float64)
        m = np.ascontiguousarray(tree.Masses[:n], dtype=np.float64)
        h = np.ascontiguousarray(tree.Softenings[:n], dtype=np.float64)
        h32 = h.astype(np.float32).astype(np.float64)
        if isinstance(tree, Octree) and np.array_equal(pos, pos32) and np.array_equal(h, h32):
            self._tree = tree  # already on the device with float32-exact positions
        else:
            self._tree = Octree(np.ascontiguousarray(pos32), m, h32, quadrupole=False)
        self.npart = n
        self.threads_x = int(threads_x)
        nodes = int(self._tree.node_hi) - n
        # arena bytes on the device: per element coordinates, mass, size, delta, softening, links
        self.device_bytes = (n + nodes) * (3 * 8 + 4 * 8 + 2 * 8)

    def _run(self, pos, softening, G, theta, group_size):
        pos = _f32(pos, (-1, 3))
        n = pos.shape[0]
        soft = _soft32(softening, n)
        res = self._tree.fields(pos.astype(np.float64), soft.astype(np.float64),
                                potential=self._KEY == "potential", accel=self._KEY == "accel", quadrupole=False,
                                group_size=group_size, theta=float(theta), G=1.0, order="morton",
                                precision="fp32")[self._KEY]
        out = res.astype(np.float32)
        return G * out


class CudaPotential(_CudaGravity):
    """Monopole gravitational potential on the GPU against one uploaded tree (cuda.py:592-600).

    float32 results. Hold the instance and call it repeatedly: the upload is the fixed cost.
    group_size (extension): targets per walk group; 1, the default, is pytreegrav.cuda's per-target
    opening test, larger groups open a superset of nodes (more accurate, faster).
    """

    _WIDTH = 1
    _KEY = "potential"

    def __call__(self, pos, softening=None, G=1.0, theta=0.7, *, group_size=1):
        """Potential at ``pos``; ``softening`` is the per-target softening (scalar or array)."""
        return self._run(pos, softening, G, theta, group_size)


class CudaAccel(_CudaGravity):
    """Monopole gravitational acceleration on the GPU against one uploaded tree (cuda.py:603-611).

    float32 results, shape (N, 3). group_size as for CudaPotential.
    """

    _WIDTH = 3
    _KEY = "accel"

    def __call__(self, pos, softening=None, G=1.0, theta=0.7, *, group_size=1):
        """Acceleration at ``pos``, shape (N, 3)."""
        return self._run(pos, softening, G, theta, group_size)


class _CudaBruteforce:
    """Shared base of the exact direct-summation contexts: the source particles go to the GPU once
    (cuda.py:737-775)."""

    _FIELD = _lib.TG_FIELD_POTENTIAL
    _WIDTH = 1

    def __init__(self, pos, m, softening=None):
        _require_device()
        pos = _f32(pos, (-1, 3))
        n = pos.shape[0]
        soft = _soft32(softening, n)
        m = _f32(m, (n,))
        self._L = _lib.load()
        self._h = ctypes.c_void_p()
        p64, m64, h64 = (np.ascontiguousarray(a.astype(np.float64)) for a in (pos, m, soft))
        _lib.check(self._L.tg_sources_create(_lib.ptr(p64), _lib.ptr(m64), _lib.ptr(h64), n, _lib.TG_MEM_HOST, None,
                                             ctypes.byref(self._h)), "source upload")
        self.n_src = n
        self.device_bytes = 8 * 5 * n

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.tg_sources_free(h)
            except Exception:
                pass
            self._h = None

    def _run(self, pos, softening, G):
        if pos is None:  # the sources themselves, self terms dropped by r == 0
            n = self.n_src
            pt = ht = None
        else:
            pos = _f32(pos, (-1, 3))
            n = pos.shape[0]
            pt = np.ascontiguousarray(pos.astype(np.float64))
            ht = np.ascontiguousarray(_soft32(softening, n).astype(np.float64))
        out = np.empty((n, self._WIDTH))
        if n:
            _lib.check(self._L.tg_sources_bruteforce(self._h, _lib.ptr(pt), _lib.ptr(ht), n, self._FIELD, 1.0,
                                                     _lib.TG_FP32, _lib.TG_MEM_HOST, _lib.ptr(out), None),
                       "bruteforce")
        out = out.astype(np.float32)
        if self._WIDTH == 1:
            out = out[:, 0]
        return G * out


class CudaPotentialBruteforce(_CudaBruteforce):
    """Exact direct-summation potential on the GPU against one uploaded source set
    (cuda.py:778-787). Targets default to the sources: the self-potential, self term excluded."""

    _FIELD = _lib.TG_FIELD_POTENTIAL
    _WIDTH = 1

    def __call__(self, pos=None, softening=None, G=1.0):
        return self._run(pos, softening, G)


class CudaAccelBruteforce(_CudaBruteforce):
    """Exact direct-summation acceleration on the GPU (cuda.py:790-796); see CudaPotentialBruteforce."""

    _FIELD = _lib.TG_FIELD_ACCEL
    _WIDTH = 3

    def __call__(self, pos=None, softening=None, G=1.0):
        return self._run(pos, softening, G)


class CudaColumnDensity:
    """Ray-traced column density on the GPU against one uploaded tree (cuda.py:240-296): the tree
    stays on the device, each call walks it for new targets and rays. float32 results, shape
    (len(pos), len(rays)); the walk itself is FP64 (tg_tree_column_density)."""

    def __init__(self, tree, threads_x=THREADS_X):
        _require_device()
        if isinstance(tree, Octree):
            self._tree = tree
        else:  # any object with pytreegrav's Octree attributes
            n = int(tree.NumParticles)
            self._tree = Octree(np.ascontiguousarray(tree.Coordinates[:n], dtype=np.float64),
                                np.ascontiguousarray(tree.Masses[:n], dtype=np.float64),
                                np.ascontiguousarray(tree.Softenings[:n], dtype=np.float64))
        self.npart = int(self._tree.NumParticles)
        self.threads_x = int(threads_x)
        nodes = int(self._tree.node_hi) - self.npart
        self.device_bytes = (self.npart + nodes) * (3 * 8 + 4 * 8 + 2 * 8)

    def __call__(self, pos, rays):
        """Column densities, shape (len(pos), len(rays)), float32; rays are normalised here."""
        pos = np.ascontiguousarray(np.atleast_2d(np.asarray(pos, dtype=np.float64)))
        rays = np.atleast_2d(np.asarray(rays, dtype=np.float64))
        rays = np.ascontiguousarray(rays / np.linalg.norm(rays, axis=1)[:, None])
        return self._tree.column_density(pos, rays).astype(np.float32)
