"""ctypes front end of the CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg as the checker or the timed CPU reference. The
product package ``pipeline_gb300`` never imports it.

``build()`` compiles oracle.c with gcc (-O2 -fopenmp -ffp-contract=off) into
oracle/_build/liboracle.so. ``load_ref()`` opens oracle/_ref/libref.so, the
reference's own sources built by oracle/build_ref.sh, when it exists.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")

# OctNode: int children[8]; vec4 corner; float cell_size; int node_mask; int leaf_mask
OCTNODE_DTYPE = np.dtype(
    [
        ("children", "<i4", (8,)),
        ("corner", "<f4", (4,)),
        ("cell_size", "<f4"),
        ("child_node_mask", "<i4"),
        ("child_leaf_mask", "<i4"),
    ]
)
assert OCTNODE_DTYPE.itemsize == 60

_lock = threading.Lock()
_lib = None
_ref = None

P = C.c_void_p


def build(force: bool = False) -> str:
    """Compile oracle.c into oracle/_build/liboracle.so (idempotent)."""
    src = os.path.join(HERE, "oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_ref(reference_root: str = "/root/reference") -> str | None:
    """Build oracle/_ref/libref.so from the reference sources, if present."""
    if not os.path.isdir(os.path.join(reference_root, "kernels")):
        return None
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), reference_root], check=True)
    return REF_PATH if os.path.exists(REF_PATH) else None


def _bind(lib):
    sig = {
        "orc_set_threads": (None, [C.c_int]),
        "orc_max_threads": (C.c_int, []),
        "orc_init_random_vec4": (None, [P, C.c_int, C.c_float, C.c_float, C.c_int]),
        "orc_morton": (None, [P, P, C.c_long, C.c_float, C.c_float]),
        "orc_radix_sort": (None, [P, C.c_int]),
        "orc_count_unique": (C.c_int, [P, C.c_int]),
        "orc_build_radix_tree": (None, [C.c_int, P, P, P, P, P, P]),
        "orc_build_radix_tree_par": (None, [C.c_int, P, P, P, P, P, P]),
        "orc_edge_count": (None, [P, P, P, C.c_int]),
        "orc_partial_sum": (None, [P, C.c_long, C.c_long, P]),
        "orc_oct_node_count": (C.c_int, [P, P, C.c_int]),
        "orc_root_init": (None, [P, P, P, C.c_float, C.c_float]),
        "orc_make_oct_nodes": (None, [P, P, P, P, P, P, C.c_float, C.c_float, C.c_int]),
        "orc_make_oct_nodes_par": (None, [P, P, P, P, P, P, C.c_float, C.c_float, C.c_int]),
        "orc_link_leaf_nodes": (None, [P, P, P, P, P, P, P, P, P, C.c_int]),
        "orc_link_leaf_nodes_par": (None, [P, P, P, P, P, P, P, P, P, C.c_int]),
        "orc_build_all": (C.c_int, [P, C.c_int, C.c_float, C.c_float, C.c_int, P, P, P, P, P, P,
                                    P, P, P, P, P, C.c_int, P]),
        "orc_fnv1a64": (C.c_uint64, [P, C.c_size_t]),
        "orc_o7_walks": (C.c_int, [P, P, P, P, C.c_int]),
        "orc_init_random_vec4_gpu": (None, [P, C.c_int, C.c_float, C.c_float, C.c_int]),
        "orc_morton_decode": (None, [P, C.c_long, C.c_float, C.c_float, P]),
        "orc_check_tree": (None, [P, C.c_int, P, C.c_int, C.c_uint32, C.c_int, C.c_int, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = _bind(C.CDLL(LIB_PATH))
    return _lib


def load_ref():
    """The reference's own CPU kernels (oracle/_ref/libref.so) or None."""
    global _ref
    with _lock:
        if _ref is None and os.path.exists(REF_PATH):
            r = C.CDLL(REF_PATH)
            sig = {
                "ref_set_threads": (None, [C.c_int]),
                "ref_init_random_vec4": (None, [P, C.c_int, C.c_float, C.c_float, C.c_int]),
                "ref_init_descending": (None, [P, C.c_int]),
                "ref_init_ascending": (None, [P, C.c_int]),
                "ref_morton": (None, [P, P, C.c_long, C.c_float, C.c_float]),
                "ref_radix_sort": (None, [P, C.c_int]),
                "ref_radix_sort_alt": (None, [P, P, C.c_int]),
                "ref_sort_inplace": (None, [P, C.c_int]),
                "ref_count_unique": (C.c_int, [P, C.c_int]),
                "ref_build_radix_tree": (None, [C.c_int, P, P, P, P, P, P]),
                "ref_edge_count": (None, [P, P, P, C.c_int]),
                "ref_partial_sum": (None, [P, C.c_long, C.c_long, P]),
                "ref_root_init": (None, [P, P, P, C.c_float, C.c_float]),
                "ref_make_oct_nodes": (None, [P, P, P, P, P, P, C.c_float, C.c_float, C.c_int]),
                "ref_link_leaf_nodes": (None, [P, P, P, P, P, P, P, P, P, C.c_int]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(r, name)
                fn.restype = res
                fn.argtypes = args
            _ref = r
    return _ref


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def fnv1a64(a: np.ndarray) -> str:
    a = np.ascontiguousarray(a)
    return "%016x" % lib().orc_fnv1a64(_p(a), a.nbytes)


# ---------------------------------------------------------------- stages --
def init_random_vec4(n: int, min_coord: float = 0.0, rng: float = 1024.0, seed: int = 114514):
    out = np.empty((n, 4), np.float32)
    lib().orc_init_random_vec4(_p(out), n, min_coord, rng, seed)
    return out


def init_random_vec4_gpu(n: int, min_coord: float = 0.0, rng: float = 1024.0, seed: int = 114514):
    """The reference's device generator, element by element (see oracle.c)."""
    out = np.empty((max(n, 0), 4), np.float32)
    if n > 0:
        lib().orc_init_random_vec4_gpu(_p(out), n, min_coord, rng, seed)
    return out


def morton_decode(codes: np.ndarray, min_coord: float, rng: float) -> np.ndarray:
    c = np.ascontiguousarray(codes, np.uint32)
    out = np.empty((len(c), 4), np.float32)
    if len(c):
        lib().orc_morton_decode(_p(c), len(c), min_coord, rng, _p(out))
    return out


def check_tree(nodes: np.ndarray, codes: np.ndarray, prefix: int, code_len: int, root: int = 0):
    """checkTree counts: (visited, leaf_checks, mismatches, rejected)."""
    nd = np.ascontiguousarray(nodes, OCTNODE_DTYPE)
    c = np.ascontiguousarray(codes, np.uint32)
    out = np.zeros(4, np.int64)
    lib().orc_check_tree(_p(nd) if len(nd) else None, len(nd), _p(c) if len(c) else None, len(c),
                         prefix, code_len, root, _p(out))
    return tuple(int(v) for v in out)


def morton(points: np.ndarray, min_coord: float, rng: float, threads: int = 1) -> np.ndarray:
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    out = np.empty(len(pts), np.uint32)
    lib().orc_set_threads(threads)
    lib().orc_morton(_p(pts), _p(out), len(pts), min_coord, rng)
    return out


def radix_sort(keys: np.ndarray, threads: int = 1) -> np.ndarray:
    k = np.array(keys, np.uint32, copy=True)
    lib().orc_set_threads(threads)
    lib().orc_radix_sort(_p(k), len(k))
    return k


def count_unique(keys: np.ndarray):
    """Returns (keys after in-place unique, U) exactly as k_CountUnique leaves them."""
    k = np.array(keys, np.uint32, copy=True)
    u = lib().orc_count_unique(_p(k), len(k))
    return k, u


def build_radix_tree(codes: np.ndarray, n_nodes: int):
    """k_BuildRadixTree(n_nodes, codes, ...) on zeroed outputs (O4)."""
    codes = np.ascontiguousarray(codes, np.uint32)
    assert len(codes) >= n_nodes + 1
    m = max(n_nodes, 1)
    prefix = np.zeros(m, np.uint8)
    hll = np.zeros(m, np.uint8)
    hlr = np.zeros(m, np.uint8)
    left = np.zeros(m, np.int32)
    parent = np.zeros(m, np.int32)
    lib().orc_build_radix_tree(n_nodes, _p(codes), _p(prefix), _p(hll), _p(hlr), _p(left), _p(parent))
    return dict(prefix_n=prefix[:n_nodes], has_leaf_left=hll[:n_nodes], has_leaf_right=hlr[:n_nodes],
                left_child=left[:n_nodes], parent=parent[:n_nodes])


def edge_count(prefix_n: np.ndarray, parent: np.ndarray) -> np.ndarray:
    n = len(prefix_n)
    ec = np.zeros(max(n, 1), np.int32)
    lib().orc_edge_count(_p(np.ascontiguousarray(prefix_n, np.uint8)), _p(np.ascontiguousarray(parent, np.int32)),
                         _p(ec), n)
    return ec[:n]


def partial_sum(data: np.ndarray) -> np.ndarray:
    d = np.ascontiguousarray(data, np.int32)
    out = np.zeros(max(len(d), 1), np.int32)
    lib().orc_partial_sum(_p(d), 0, len(d), _p(out))
    return out[: len(d)]


def oct_node_count(ec: np.ndarray, ps: np.ndarray) -> int:
    return lib().orc_oct_node_count(_p(np.ascontiguousarray(ec, np.int32)), _p(np.ascontiguousarray(ps, np.int32)), len(ec))


def o7_walks(ec, has_leaf_left, has_leaf_right, parent) -> int:
    """Count LinkLeaf walks that reach radix node 0 (contract O7 inputs)."""
    return lib().orc_o7_walks(_p(np.ascontiguousarray(ec, np.int32)), _p(np.ascontiguousarray(has_leaf_left, np.uint8)),
                              _p(np.ascontiguousarray(has_leaf_right, np.uint8)),
                              _p(np.ascontiguousarray(parent, np.int32)), len(ec))


def make_octree(codes, tree, ec, ps, min_coord, rng, n_oct=None):
    """Root set-up + k_MakeOctNodes + k_LinkLeafNodes, sequential (O6)."""
    B = len(ec)
    if n_oct is None:
        n_oct = oct_node_count(ec, ps)
    nodes = np.zeros(max(n_oct, 1), OCTNODE_DTYPE)
    codes = np.ascontiguousarray(codes, np.uint32)
    L = lib()
    L.orc_root_init(_p(nodes), _p(codes), _p(tree["prefix_n"]), min_coord, rng)
    L.orc_make_oct_nodes(_p(nodes), _p(ps), _p(ec), _p(codes), _p(tree["prefix_n"]), _p(tree["parent"]),
                         min_coord, rng, B)
    L.orc_link_leaf_nodes(_p(nodes), _p(ps), _p(ec), _p(codes), _p(tree["has_leaf_left"]),
                          _p(tree["has_leaf_right"]), _p(tree["prefix_n"]), _p(tree["parent"]),
                          _p(tree["left_child"]), B)
    return nodes[:n_oct]


def build_all(points: np.ndarray, min_coord: float, rng: float, threads: int = 1,
              parallel_octree: bool = False, keep_morton: bool = True):
    """Whole build (apps/cpu_demo/main.cpp:72-154 order, contract O1-O11).

    Returns a dict with every stage buffer plus per-stage wall times (ms).
    """
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    n = len(pts)
    m = max(n, 1)
    morton_out = np.empty(m, np.uint32) if keep_morton else None
    keys = np.empty(m, np.uint32)
    nu = C.c_int(0)
    prefix = np.zeros(m, np.uint8)
    hll = np.zeros(m, np.uint8)
    hlr = np.zeros(m, np.uint8)
    left = np.zeros(m, np.int32)
    parent = np.zeros(m, np.int32)
    ec = np.zeros(m, np.int32)
    ps = np.zeros(m, np.int32)
    cap = max(n, 16)
    stage_ms = np.zeros(8, np.float64)
    L = lib()
    L.orc_set_threads(threads)
    while True:
        nodes = np.empty(cap, OCTNODE_DTYPE)
        M = L.orc_build_all(_p(pts), n, min_coord, rng, int(parallel_octree),
                            _p(morton_out) if keep_morton else None, _p(keys), C.byref(nu), _p(prefix),
                            _p(hll), _p(hlr), _p(left), _p(parent), _p(ec), _p(ps), _p(nodes), cap,
                            _p(stage_ms))
        if M >= 0:
            break
        cap = -M
    U = nu.value
    B = max(U - 1, 0)
    out = dict(
        n_unique=U, n_brt=B, n_oct=M, sorted_unique=keys[:U].copy(), keys_after_unique=keys[:n].copy(),
        prefix_n=prefix[:B], has_leaf_left=hll[:B], has_leaf_right=hlr[:B], left_child=left[:B],
        parent=parent[:B], edge_count=ec[:B], prefix_sum=ps[:B], oct_nodes=nodes[:M],
        stage_ms=stage_ms,
    )
    if keep_morton:
        out["morton"] = morton_out[:n]
    return out
