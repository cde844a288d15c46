"""ctypes binding of libpytreegrav_gb300.so (the C ABI in include/pytreegrav_gb300.h).

The library is built in-tree (pytreegrav_gb300/_build/) by pytreegrav_gb300.build. There is no CPU
fallback: if the library is missing or cannot run, every compute call raises.
"""

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpytreegrav_gb300.so")

TG_OK = 0
TG_ERR_BAD_ARG = 1
TG_ERR_NONFINITE = 2
TG_ERR_OOM = 3
TG_ERR_STACK_OVERFLOW = 4
TG_ERR_ITER_LIMIT = 5
TG_ERR_QUEUE_TIMEOUT = 6
TG_ERR_CUDA = 7
TG_ERR_NO_QUADRUPOLES = 8

TG_MEM_HOST = 0
TG_MEM_DEVICE = 1
TG_FIELD_POTENTIAL = 1
TG_FIELD_ACCEL = 2
TG_FIELD_TIDAL = 4
TG_FP32 = 0
TG_FP64 = 1
TG_ORDER_TREE = 0
TG_ORDER_MORTON = 1
TG_ORDER_GIVEN = 2
TG_GROUP_BLOCKS = 0
TG_GROUP_TREE = 1
TG_NOALLOC_MAX_POINTS = 262144
TG_CORR_KINDS = {"density": 0, "velocity": 1, "structure": 2}
TG_CORR_MAX_BINS = 4096

# every extern "C" symbol declared in include/pytreegrav_gb300.h
EXPORTS = [
    "tg_last_error",
    "tg_tree_build",
    "tg_tree_build_batched",
    "tg_tree_info_get",
    "tg_tree_quadrupoles",
    "tg_tree_copy_out",
    "tg_tree_free",
    "tg_tree_fields",
    "tg_targets_create",
    "tg_targets_free",
    "tg_targets_info",
    "tg_targets_groups_copy",
    "tg_targets_fields",
    "tg_tree_last_walk_stats",
    "tg_tree_set_walk_config",
    "tg_walk_graph_create",
    "tg_walk_graph_launch",
    "tg_walk_graph_status",
    "tg_walk_graph_free",
    "tg_morton_order",
    "tg_morton_order_noalloc",
    "tg_bruteforce",
    "tg_tree_column_density",
    "tg_tree_set_velocities",
    "tg_tree_copy_velocities",
    "tg_tree_correlation",
    "tg_device_count",
    "tg_sources_create",
    "tg_sources_bruteforce",
    "tg_sources_free",
]

# every extern "C" symbol declared in include/pytreegrav_gb300_theta.h
THETA_EXPORTS = [
    "tg_tree_groups",
    "tg_tree_groups_copy",
    "tg_tree_record_group_stats",
    "tg_tree_last_group_stats",
    "tg_tree_last_group_error",
    "tg_theta_features",
    "tg_mlp_forward",
    "tg_mlp_backward",
    "tg_adam_step",
    "tg_theta_loss",
    "tg_theta_tolerances",
    "tg_theta_model_create",
    "tg_theta_model_free",
    "tg_theta_model_set_error_budget",
    "tg_theta_infer",
    "tg_tree_fields_grouped",
    "tg_tree_fields_learned",
    "tg_targets_fields_learned",
    "tg_targets_features",
    "tg_targets_tolerances",
]
# every extern "C" symbol declared in include/pytreegrav_gb300_measure.h (measurement and self-checks)
MEASURE_EXPORTS = [
    "tg_tree_last_walk_steps",
    "tg_tree_last_walk_quad_interactions",
    "tg_tree_last_walk_kernel_ms",
    "tg_launch_count",
    "tg_measure_fp32_fma",
    "tg_check_f32_conversion",
    "tg_set_loop_limits",
]
TG_THETA_NFEAT = 16
TG_MLP_H = 64
TG_MLP_NPARAM = TG_MLP_H * TG_THETA_NFEAT + TG_MLP_H + TG_MLP_H * TG_MLP_H + TG_MLP_H + TG_MLP_H + 1
TG_THETA_FEAT_LAMBDA = 13
TG_THETA_KIND_ANGLE = 0
TG_THETA_KIND_TOLERANCE = 1


class TreeInfo(ctypes.Structure):
    _fields_ = [
        ("npart", ctypes.c_int64),
        ("num_nodes", ctypes.c_int64),
        ("node_hi", ctypes.c_int64),
        ("has_quads", ctypes.c_int32),
        ("has_coincident", ctypes.c_int32),
        ("n_systems", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("coord", ctypes.c_void_p),
        ("mass", ctypes.c_void_p),
        ("size", ctypes.c_void_p),
        ("delta", ctypes.c_void_p),
        ("soft", ctypes.c_void_p),
        ("quad", ctypes.c_void_p),
        ("first", ctypes.c_void_p),
        ("next", ctypes.c_void_p),
        ("walk_idx", ctypes.c_void_p),
    ]


class GravityError(RuntimeError):
    """A device-side failure reported by the library (CUDA error, stack overflow, ...)."""


_lib = None
_lock = threading.Lock()


def _declare(L):
    vp, i64, i32, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_double
    ci = ctypes.c_int
    L.tg_last_error.argtypes = []
    L.tg_last_error.restype = ctypes.c_char_p
    L.tg_tree_build.argtypes = [vp, vp, vp, i64, ci, ci, ci, vp, ctypes.POINTER(vp)]
    L.tg_tree_build_batched.argtypes = [vp, vp, vp, vp, i32, ci, ci, vp, ctypes.POINTER(vp)]
    L.tg_tree_info_get.argtypes = [vp, ctypes.POINTER(TreeInfo)]
    L.tg_tree_quadrupoles.argtypes = [vp, ctypes.POINTER(vp), vp]
    L.tg_tree_copy_out.argtypes = [vp] * 10 + [vp]
    L.tg_tree_free.argtypes = [vp]
    L.tg_tree_fields.argtypes = [vp, vp, vp, i64, ci, ci, dbl, dbl, ci, ci, ci, ci, vp, ci, vp, vp]
    L.tg_tree_last_walk_stats.argtypes = [vp, vp, vp, vp, vp]
    L.tg_targets_create.argtypes = [vp, vp, vp, i64, ci, ci, vp, ctypes.POINTER(vp)]
    L.tg_targets_free.argtypes = [vp]
    L.tg_targets_info.argtypes = [vp, vp, vp]
    L.tg_targets_groups_copy.argtypes = [vp, vp, vp, vp, vp, ci, vp]
    L.tg_targets_fields.argtypes = [vp, ci, ci, dbl, dbl, ci, vp, ci, vp, vp]
    L.tg_tree_set_walk_config.argtypes = [vp, ci, ci]
    L.tg_walk_graph_create.argtypes = [vp, ci, ci, dbl, dbl, ci, ci, vp, ctypes.POINTER(vp)]
    L.tg_walk_graph_launch.argtypes = [vp, vp]
    L.tg_walk_graph_status.argtypes = [vp, vp]
    L.tg_walk_graph_free.argtypes = [vp]
    L.tg_morton_order.argtypes = [vp, i64, ci, vp, vp]
    L.tg_morton_order_noalloc.argtypes = [vp, i64, vp, vp]
    L.tg_bruteforce.argtypes = [vp, vp, i64, vp, vp, vp, i64, ci, ci, dbl, ci, ci, vp, vp]
    L.tg_tree_column_density.argtypes = [vp, vp, i64, vp, i64, i64, ci, dbl, ci, ci, vp, vp]
    L.tg_tree_set_velocities.argtypes = [vp, vp, ci, vp]
    L.tg_tree_copy_velocities.argtypes = [vp, vp, vp, vp]
    L.tg_tree_correlation.argtypes = [vp, ci, vp, vp, vp, i64, vp, ci, dbl, dbl, dbl, ci, ctypes.c_uint64, ci, vp,
                                      vp, vp]
    L.tg_device_count.argtypes = [ctypes.POINTER(ci)]
    L.tg_sources_create.argtypes = [vp, vp, vp, i64, ci, vp, ctypes.POINTER(vp)]
    L.tg_sources_bruteforce.argtypes = [vp, vp, vp, i64, ci, dbl, ci, ci, vp, vp]
    L.tg_sources_free.argtypes = [vp]
    for name in EXPORTS[1:]:
        getattr(L, name).restype = ci
    flt = ctypes.c_float
    L.tg_tree_groups.argtypes = [vp, ci, vp, vp]
    L.tg_tree_groups_copy.argtypes = [vp, ci, vp, vp, vp, ci, vp]
    L.tg_tree_record_group_stats.argtypes = [vp, ci]
    L.tg_tree_last_group_stats.argtypes = [vp, vp, ci, vp]
    L.tg_theta_features.argtypes = [vp, ci, ci, vp, vp]
    L.tg_mlp_forward.argtypes = [vp, vp, i64, vp, vp, vp]
    L.tg_mlp_backward.argtypes = [vp, vp, vp, vp, i64, vp, vp, vp]
    L.tg_adam_step.argtypes = [vp, vp, vp, vp, i64, flt, flt, flt, flt, ci, vp]
    L.tg_theta_loss.argtypes = [vp, vp, vp, vp, i64, ci, flt, flt, flt, flt, vp, vp, vp]
    L.tg_theta_tolerances.argtypes = [vp, ci, ci, vp, vp, vp]
    L.tg_theta_model_create.argtypes = [vp, vp, vp, ci, flt, flt, flt, ci, ctypes.POINTER(vp)]
    L.tg_theta_model_free.argtypes = [vp]
    L.tg_theta_model_set_error_budget.argtypes = [vp, flt]
    L.tg_tree_last_group_error.argtypes = [vp, vp, ci, vp]
    L.tg_theta_infer.argtypes = [vp, vp, i64, flt, vp, vp]
    L.tg_tree_fields_grouped.argtypes = [vp, ci, ci, dbl, ci, dbl, vp, vp, ci, vp, vp]
    L.tg_tree_fields_learned.argtypes = [vp, ci, ci, dbl, ci, vp, flt, dbl, ci, vp, vp]
    L.tg_targets_fields_learned.argtypes = [vp, ci, ci, dbl, vp, flt, dbl, ci, vp, vp]
    L.tg_targets_features.argtypes = [vp, ci, vp, vp]
    L.tg_targets_tolerances.argtypes = [vp, ci, vp, vp, vp]
    for name in THETA_EXPORTS:
        getattr(L, name).restype = ci


def load(path=None):
    """Load (once) and return the library; raises if it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            p = path or LIB_PATH
            if not os.path.exists(p):
                raise GravityError(
                    f"pytreegrav_gb300: the CUDA library {p} is not built; run "
                    "`python -m pytreegrav_gb300.build` (needs nvcc).")
            L = ctypes.CDLL(p)
            _declare(L)
            _lib = L
    return _lib


NONFINITE_MSG = "Invalid input detected - aborting treebuild to avoid going into an infinite loop!"


class NonFiniteInput(RuntimeError):
    """TG_ERR_NONFINITE: a position, mass or softening is NaN or infinite (ConstructTree's error,
    frontend.py:123-125)."""


def check(rc, what=""):
    if rc == TG_OK:
        return
    L = load()
    msg = f"{what}: " if what else ""
    if rc == TG_ERR_BAD_ARG:
        raise ValueError(msg + "invalid argument")
    if rc == TG_ERR_NONFINITE:
        raise NonFiniteInput(msg + NONFINITE_MSG)
    if rc == TG_ERR_OOM:
        raise MemoryError(msg + "device allocation failed")
    if rc == TG_ERR_NO_QUADRUPOLES:
        raise ValueError(
            "quadrupole=True requires a tree built with quadrupole moments: pass a tree from "
            "ConstructTree(..., quadrupole=True), or evaluate with quadrupole=False.")
    if rc == TG_ERR_STACK_OVERFLOW:
        raise GravityError(msg + "tree walk node stack overflowed (result not written)")
    if rc == TG_ERR_CUDA:
        raise GravityError(msg + "CUDA error: " + (L.tg_last_error() or b"").decode())
    raise GravityError(msg + f"status {rc}")


def ptr(a):
    """Host pointer of a C-contiguous numpy array (or None)."""
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data)
