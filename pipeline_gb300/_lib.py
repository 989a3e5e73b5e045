"""ctypes binding of libpipeline_gb300.so (the C ABI in include/octree_gb300.h).

The library is the only compute path: if it is missing this module raises
instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

LIB_PATH = _build.LIB_PATH

OCT_OK = 0
OCT_ERR_INVALID_ARG = 1
OCT_ERR_WORKSPACE = 2
OCT_ERR_CUDA = 3
OCT_ERR_DEVICE = 4
OCT_ERR_CAPACITY = 5
OCT_ERR_TOO_LARGE = 6

OCT_STATUS_SPIN_TIMEOUT = 1
OCT_STATUS_WALK_LIMIT = 2
OCT_STATUS_RANGE = 4
OCT_STATUS_CAPACITY = 8

OCT_MAX_N = (1 << 30) - 1

OCT_DIAG_WAIT_SORT = 0
OCT_DIAG_WAIT_SCAN = 1

_STATUS_NAMES = {
    OCT_ERR_INVALID_ARG: "invalid argument",
    OCT_ERR_WORKSPACE: "workspace too small",
    OCT_ERR_CUDA: "CUDA error",
    OCT_ERR_DEVICE: "device status set",
    OCT_ERR_CAPACITY: "octree capacity too small",
}

P = C.c_void_p
I = C.c_int
F = C.c_float
Z = C.c_size_t


class OctError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        msg = f"{where}: {_STATUS_NAMES.get(code, code)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


class OctBuildOutputs(C.Structure):
    """oct_build_outputs (include/octree_gb300.h)."""

    _fields_ = [
        ("codes", P),
        ("n_nodes", C.c_int32),
        ("prefix_n", P),
        ("has_leaf_left", P),
        ("has_leaf_right", P),
        ("left_child", P),
        ("parent", P),
        ("edge_count", P),
        ("prefix_sum", P),
        ("nodes", P),
        ("nodes_capacity", C.c_int32),
        ("d_counts", P),
    ]


# name -> (restype, argtypes). Every entry is a declaration of include/octree_gb300.h.
SIGNATURES = {
    "oct_version": (I, []),
    "oct_built_arch": (I, []),
    "oct_last_error": (C.c_char_p, []),
    "oct_init_random_vec4": (None, [P, I, F, F, I]),
    "oct_morton_encode": (I, [P, P, C.c_int64, F, F, P, P]),
    "oct_sort_workspace_bytes": (Z, [I, I]),
    "oct_sort_keys": (I, [P, P, I, I, P, Z, P, P]),
    "oct_sort_keys_noalloc": (I, [P, P, I, I, P, P]),
    "oct_unique_workspace_bytes": (Z, [I]),
    "oct_unique": (I, [P, I, P, P, Z, P, P]),
    "oct_build_radix_tree": (I, [I, P, P, P, P, P, P, P]),
    "oct_radix_tree_sorted_workspace_bytes": (Z, [I]),
    "oct_build_radix_tree_sorted": (I, [I, P, P, P, P, P, P, P, P, Z, P]),
    "oct_edge_count": (I, [P, P, P, I, P]),
    "oct_prefix_sum_workspace_bytes": (Z, [I]),
    "oct_prefix_sum": (I, [P, I, P, P, Z, P, P]),
    "oct_octree_node_count": (I, [P, P, I, P, P]),
    "oct_octree_workspace_bytes": (Z, [I]),
    "oct_octree_root_init": (I, [P, P, P, F, F, P]),
    "oct_make_oct_nodes": (I, [P, I, P, P, P, P, P, F, F, I, P, Z, P, P]),
    "oct_link_leaf_nodes": (I, [P, I, P, P, P, P, P, P, P, P, I, P, Z, P, P]),
    "oct_build_workspace_bytes": (Z, [I, I]),
    "oct_build_octree": (I, [P, I, F, F, C.POINTER(OctBuildOutputs), P, Z, P]),
    "oct_read_counts": (I, [P, P, P]),
    "oct_init_descending": (I, [P, I, P]),
    "oct_init_ascending": (I, [P, I, P]),
    "oct_init_random_vec4_device": (I, [P, I, F, F, I, P]),
    "oct_morton_decode": (I, [P, I, F, F, P, P]),
    "oct_check_tree_workspace_bytes": (Z, [I]),
    "oct_check_tree": (I, [P, I, P, I, C.c_uint32, I, I, P, P, Z, P]),
    "oct_lcdf_layout": (I, [I, P]),
    "oct_lcdf_fit_workspace_bytes": (Z, [I]),
    "oct_lcdf_fit": (I, [P, I, I, I, F, I, P, I, P, Z, P]),
    "oct_lcdf_loss_grad": (I, [P, I, P, I, P, P]),
    "oct_lcdf_tables": (I, [P, I, I, P]),
    "oct_lcdf_train_steps": (I, [P, I, P, I, I, F, P]),
    "oct_lcdf_buckets": (I, [P, I, P, I, P, P]),
    "oct_lsort_workspace_bytes": (Z, [I, I, I]),
    "oct_lsort_unique": (I, [P, I, P, I, I, F, P, P, P, P, Z, P, P]),
    "oct_build_learned_workspace_bytes": (Z, [I, I, I, I]),
    "oct_build_octree_learned": (I, [P, I, F, F, P, I, I, F, C.POINTER(OctBuildOutputs), P, P, Z, P]),
    "oct_set_sort_config": (I, [I, I, I, I]),
    "oct_get_sort_config": (I, [P]),
    "oct_batch_plan_create": (P, [I, P, P]),
    "oct_batch_plan_destroy": (None, [P]),
    "oct_batch_plan_info": (I, [P, P]),
    "oct_batch_upload_tables": (I, [P, P, P]),
    "oct_build_octree_batch": (I, [P, P, P, P, P, C.POINTER(OctBuildOutputs), P, P, Z, P]),
    "oct_batch_learned_workspace_bytes": (Z, [P, I]),
    "oct_set_batch_work_queue": (I, [I]),
    "oct_build_octree_batch_learned": (I, [P, P, P, P, P, P, I, I, C.POINTER(OctBuildOutputs), P,
                                           P, P, Z, P]),
    "oct_build_sort_form": (I, [P, I, I, P]),
    "oct_build_step_count": (I, []),
    "oct_build_step_name": (C.c_char_p, [I]),
    "oct_build_octree_timed": (I, [P, I, F, F, C.POINTER(OctBuildOutputs), P, Z, P, I, P]),
    "oct_diag_wait_workspace_bytes": (Z, []),
    "oct_diag_lookback_timeout": (I, [I, C.c_ulonglong, P, Z, P, P]),
}

_lock = threading.Lock()
_lib = None


def load(build_if_missing: bool = True):
    """Load (building in-tree first if needed) and bind the native library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise ImportError(f"{LIB_PATH} is not built; run python -m pipeline_gb300.build")
            _build.build()
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int, where: str) -> None:
    if rc != OCT_OK:
        detail = load().oct_last_error().decode(errors="replace") if rc == OCT_ERR_CUDA else ""
        raise OctError(rc, where, detail)
