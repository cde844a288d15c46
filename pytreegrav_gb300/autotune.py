"""Autotuner for the tree walk's launch shape (no counterpart in pytreegrav).

Three knobs set how a walk maps onto the GPU: the group size (targets per traversal, 8/16/32 -- the
leaf-group size of the tree grouping), the block shape (2, 4 or 8 warps per block) and the node stack a
walk starts with (1024 entries per warp, groups that overflow it being rewalked on the device with
4096; or 4096 for every group, with fewer resident warps). Block shape and stack never change a result;
the group size changes which nodes a group accepts (larger groups accept a superset), within the
walk's accuracy. :func:`tune` times every combination on the caller's own tree with the walk kernel's
own device time, keeps the fastest, applies it to the tree, and caches it under a signature of the
workload (particle and system counts in powers of two, fields, multipole order, angle), so later trees
of the same kind reuse it without timing (:func:`apply`).

The cache is a JSON file: $TG_AUTOTUNE_CACHE, else ~/.cache/pytreegrav_gb300/autotune.json.
"""

import ctypes
import itertools
import json
import math
import os

from . import _lib

GROUP_SIZES = (8, 16, 32)
WARPS = (2, 4, 8)
STACKS = (1024, 4096)


def cache_path():
    return os.environ.get("TG_AUTOTUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "pytreegrav_gb300",
                                                              "autotune.json")


def _load_cache():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, value):
    c = _load_cache()
    c[key] = value
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(c, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def signature(n_particles, n_systems, fields, quadrupole, theta):
    return (f"n2^{round(math.log2(max(n_particles, 1)))}|sys2^{round(math.log2(max(n_systems, 1)))}"
            f"|f{int(fields)}|q{int(bool(quadrupole))}|t{round(float(theta), 2)}")


def _kernel_ms(L, h):
    L.tg_tree_last_walk_kernel_ms.restype = ctypes.c_double
    L.tg_tree_last_walk_kernel_ms.argtypes = [ctypes.c_void_p]
    return float(L.tg_tree_last_walk_kernel_ms(h))


def tune(tree, fields=_lib.TG_FIELD_ACCEL, quadrupole=False, theta=0.7, G=1.0, n_systems=1, repeats=2,
         group_sizes=GROUP_SIZES, warps=WARPS, stacks=STACKS, use_cache=True):
    """Time every (group size, warps per block, first stack) on `tree` (an Octree), apply and return
    the fastest as a dict (with the timings of all candidates under "timings", in ms)."""
    key = signature(tree.NumParticles, n_systems, fields, quadrupole, theta)
    if use_cache:
        hit = _load_cache().get(key)
        if hit:
            tree.set_walk_config(hit["warps"], hit["stack"])
            return dict(hit, cached=True)
    L = _lib.load()
    import numpy as np

    W = int(bool(fields & 1)) + 3 * int(bool(fields & 2)) + 9 * int(bool(fields & 4))
    out = np.empty((tree.NumParticles, W))
    timings = {}
    for gs, w, st in itertools.product(group_sizes, warps, stacks):
        tree.set_walk_config(w, st)
        best = float("inf")
        for _ in range(repeats):
            rc = L.tg_tree_fields(tree._h, None, None, tree.NumParticles, int(fields), int(bool(quadrupole)),
                                  float(theta), float(G), int(gs), _lib.TG_GROUP_TREE, _lib.TG_ORDER_TREE,
                                  _lib.TG_FP32, None, _lib.TG_MEM_HOST, _lib.ptr(out), None)
            _lib.check(rc, "autotune walk")
            best = min(best, _kernel_ms(L, tree._h))
        timings[f"{gs}/{w}/{st}"] = round(best, 4)
    gs, w, st = min(itertools.product(group_sizes, warps, stacks), key=lambda c: timings[f"{c[0]}/{c[1]}/{c[2]}"])
    tree.set_walk_config(w, st)
    result = {"group_size": gs, "warps": w, "stack": st, "ms": timings[f"{gs}/{w}/{st}"], "key": key}
    _store(key, result)
    return dict(result, timings=timings, cached=False)


def apply(tree, fields=_lib.TG_FIELD_ACCEL, quadrupole=False, theta=0.7, n_systems=1):
    """Apply a cached choice for this workload to `tree`; returns it, or None when nothing is cached."""
    hit = _load_cache().get(signature(tree.NumParticles, n_systems, fields, quadrupole, theta))
    if hit:
        tree.set_walk_config(hit["warps"], hit["stack"])
    return hit
