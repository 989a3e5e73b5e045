"""Reference-named stage functions on device tensors.

Each function keeps the name, argument order and meaning of the reference's
per-stage entry point (include/kernels/*.hpp of ucsc-redwood/pipeline) and
runs the sm_103a kernels of libpipeline_gb300.so on the current torch CUDA
stream. Buffers are caller-owned CUDA tensors, as the reference's buffers are
caller-owned (include/shared/types.h:5-8):

  points      float32 [n, 4]  (glm::vec4)
  keys/codes  int32   [n]     (unsigned int bit patterns)
  prefix_n, has_leaf_left, has_leaf_right  uint8 [n_nodes]
  left_child, parent, edge_count, prefix_sum int32 [n_nodes]
  oct_nodes   int32   [M, 15] (OctNode, 60 bytes; corner/cell_size as float bits)

Calls are asynchronous like CUDA launches, except those that return a host
value (k_CountUnique), which synchronise the stream first.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

OCTNODE_WORDS = 15
OCTNODE_DTYPE = np.dtype(
    [
        ("children", "<i4", (8,)),
        ("corner", "<f4", (4,)),
        ("cell_size", "<f4"),
        ("child_node_mask", "<i4"),
        ("child_leaf_mask", "<i4"),
    ]
)


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor | None, name: str, dtype=None, min_numel: int = 0) -> C.c_void_p:
    if t is None:
        return C.c_void_p(0)
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if t.numel() < min_numel:
        raise ValueError(f"{name} holds {t.numel()} elements, needs {min_numel}")
    return C.c_void_p(t.data_ptr())


def _workspace(nbytes: int, device) -> torch.Tensor:
    # 256-byte aligned (the caching allocator aligns blocks to 512 bytes).
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def oct_nodes_to_numpy(nodes: torch.Tensor) -> np.ndarray:
    """Copy an OctNode tensor [M, 15] to a host structured array."""
    a = nodes.detach().to("cpu").contiguous().numpy()
    return a.view(OCTNODE_DTYPE).reshape(-1)


def empty_oct_nodes(m: int, device="cuda") -> torch.Tensor:
    """Zeroed OctNode storage, as the oracle contract (O4) requires."""
    return torch.zeros((max(m, 0), OCTNODE_WORDS), dtype=torch.int32, device=device)


# ------------------------------------------------------------------ stage 0 --
def k_InitRandomVec4(u_data, n: int, min: float, range: float, seed: int):  # noqa: A002
    """include/kernels/00_init.hpp:10-11 (host). Fills a host float32 [n, 4]
    array or returns a new one when u_data is None."""
    if u_data is None:
        u_data = np.empty((n, 4), np.float32)
    arr = u_data.numpy() if isinstance(u_data, torch.Tensor) else u_data
    if arr.dtype != np.float32 or arr.size < 4 * n or not arr.flags["C_CONTIGUOUS"]:
        raise ValueError("u_data must be a contiguous host float32 array of n x 4")
    _lib.load().oct_init_random_vec4(arr.ctypes.data, n, min, range, seed)
    return u_data


# ------------------------------------------------------------------ stage 1 --
def k_ComputeMortonCode(data: torch.Tensor, morton_keys: torch.Tensor, n: int, min_coord: float,
                        range: float, status: torch.Tensor | None = None):  # noqa: A002
    """include/kernels/01_morton.hpp:9-13."""
    lib = _lib.load()
    _lib.check(lib.oct_morton_encode(_ptr(data, "data", torch.float32, 4 * n),
                                     _ptr(morton_keys, "morton_keys", torch.int32, n), n, min_coord,
                                     range, _ptr(status, "status"), _stream()),
               "k_ComputeMortonCode")


# ------------------------------------------------------------------ stage 2 --
def k_SimpleRadixSort(keys: torch.Tensor, a, b=None, key_bits: int = 32,
                      status: torch.Tensor | None = None):
    """include/kernels/02_sort.hpp:6-7: k_SimpleRadixSort(keys, n) or
    k_SimpleRadixSort(keys, keys_alt, n). Sorts keys[0, n) ascending in place."""
    if b is None:
        alt, n = None, int(a)
    else:
        alt, n = a, int(b)
    if n <= 1:
        return
    if alt is None:
        alt = torch.empty(n, dtype=torch.int32, device=keys.device)
    lib = _lib.load()
    ws = _workspace(lib.oct_sort_workspace_bytes(n, key_bits), keys.device)
    _lib.check(lib.oct_sort_keys(_ptr(keys, "keys", torch.int32, n),
                                 _ptr(alt, "keys_alt", torch.int32, n), n, key_bits,
                                 _ptr(ws, "workspace"), ws.numel(), _ptr(status, "status"),
                                 _stream()),
               "k_SimpleRadixSort")


def k_SortKeysInplace(keys: torch.Tensor, n: int):
    """include/kernels/02_sort.hpp:5."""
    k_SimpleRadixSort(keys, n)


# ------------------------------------------------------------------ stage 3 --
def k_CountUnique(keys: torch.Tensor, n: int, status: torch.Tensor | None = None) -> int:
    """include/kernels/03_unique.hpp:4. Compacts in place, returns U."""
    lib = _lib.load()
    d_u = torch.zeros(1, dtype=torch.int32, device=keys.device)
    ws = _workspace(lib.oct_unique_workspace_bytes(n), keys.device)
    _lib.check(lib.oct_unique(_ptr(keys, "keys", torch.int32, n), n, _ptr(d_u, "n_unique"),
                              _ptr(ws, "workspace"), ws.numel(), _ptr(status, "status"), _stream()),
               "k_CountUnique")
    return int(d_u.item())


# ------------------------------------------------------------------ stage 4 --
def k_BuildRadixTree(n: int, codes: torch.Tensor, prefix_n: torch.Tensor,
                     has_leaf_left: torch.Tensor, has_leaf_right: torch.Tensor,
                     left_child: torch.Tensor, parent: torch.Tensor):
    """include/kernels/04_radix_tree.hpp:5-11 (n = number of radix nodes = U - 1)."""
    lib = _lib.load()
    _lib.check(lib.oct_build_radix_tree(
        n, _ptr(codes, "codes", torch.int32, n + 1), _ptr(prefix_n, "prefix_n", torch.uint8, n),
        _ptr(has_leaf_left, "has_leaf_left", torch.uint8, n),
        _ptr(has_leaf_right, "has_leaf_right", torch.uint8, n),
        _ptr(left_child, "left_child", torch.int32, n), _ptr(parent, "parent", torch.int32, n),
        _stream()), "k_BuildRadixTree")


def build_radix_tree_sorted(n: int, codes: torch.Tensor, prefix_n: torch.Tensor,
                            has_leaf_left: torch.Tensor, has_leaf_right: torch.Tensor,
                            left_child: torch.Tensor, parent: torch.Tensor,
                            edge_count: torch.Tensor | None = None):
    """Stage 4 (and, with ``edge_count``, stage 5) for strictly increasing
    codes below 2^31, from the deltas of adjacent codes: the outputs of
    k_BuildRadixTree (include/kernels/04_radix_tree.hpp:5-11) and k_EdgeCount
    (include/kernels/05_edge_count.hpp:5-8) for such codes."""
    lib = _lib.load()
    ws_bytes = lib.oct_radix_tree_sorted_workspace_bytes(n)
    ws = _workspace(ws_bytes, codes.device)
    ec = _ptr(edge_count, "edge_count", torch.int32, n)
    _lib.check(lib.oct_build_radix_tree_sorted(
        n, _ptr(codes, "codes", torch.int32, n + 1), _ptr(prefix_n, "prefix_n", torch.uint8, n),
        _ptr(has_leaf_left, "has_leaf_left", torch.uint8, n),
        _ptr(has_leaf_right, "has_leaf_right", torch.uint8, n),
        _ptr(left_child, "left_child", torch.int32, n), _ptr(parent, "parent", torch.int32, n),
        ec, C.c_void_p(ws.data_ptr()), ws_bytes, _stream()), "build_radix_tree_sorted")


# ------------------------------------------------------------------ stage 5 --
def k_EdgeCount(prefix_n: torch.Tensor, parents: torch.Tensor, edge_count: torch.Tensor,
                n_brt_nodes: int):
    """include/kernels/05_edge_count.hpp:5-8."""
    lib = _lib.load()
    n = n_brt_nodes
    _lib.check(lib.oct_edge_count(_ptr(prefix_n, "prefix_n", torch.uint8, n),
                                  _ptr(parents, "parents", torch.int32, n),
                                  _ptr(edge_count, "edge_count", torch.int32, n), n, _stream()),
               "k_EdgeCount")


# ------------------------------------------------------------------ stage 6 --
def k_PartialSum(data: torch.Tensor, first: int, last: int, d_first: torch.Tensor,
                 status: torch.Tensor | None = None) -> int:
    """include/kernels/06_partial_sum.hpp:6-9: inclusive scan of data[first:last]
    into d_first[0:last-first]; returns last - first (one past the last output,
    as the reference returns a one-past-end pointer)."""
    n = int(last - first)
    if n <= 0:
        return 0
    lib = _lib.load()
    src = data[first:last]
    ws = _workspace(lib.oct_prefix_sum_workspace_bytes(n), data.device)
    _lib.check(lib.oct_prefix_sum(_ptr(src, "data", torch.int32, n), n,
                                  _ptr(d_first, "d_first", torch.int32, n), _ptr(ws, "workspace"),
                                  ws.numel(), _ptr(status, "status"), _stream()), "k_PartialSum")
    return n


def octree_node_count(edge_count: torch.Tensor, prefix_sum: torch.Tensor, n_brt_nodes: int) -> int:
    """Number of OctNodes stages 7-8 write for this tree (contract O3)."""
    lib = _lib.load()
    out = torch.zeros(1, dtype=torch.int32, device=edge_count.device)
    _lib.check(lib.oct_octree_node_count(_ptr(edge_count, "edge_count", torch.int32, n_brt_nodes),
                                         _ptr(prefix_sum, "prefix_sum", torch.int32, n_brt_nodes),
                                         n_brt_nodes, _ptr(out, "out"), _stream()),
               "octree_node_count")
    return int(out.item())


def octree_root_init(oct_nodes: torch.Tensor, codes: torch.Tensor, prefix_n: torch.Tensor,
                     min_coord: float, range: float):  # noqa: A002
    """Root set-up of apps/cpu_demo/main.cpp:125-132 on the device."""
    lib = _lib.load()
    _lib.check(lib.oct_octree_root_init(_ptr(oct_nodes, "oct_nodes", torch.int32, OCTNODE_WORDS),
                                        _ptr(codes, "codes", torch.int32, 1),
                                        _ptr(prefix_n, "prefix_n", torch.uint8, 1), min_coord, range,
                                        _stream()), "octree_root_init")


# ------------------------------------------------------------------ stage 7 --
def k_MakeOctNodes(oct_nodes: torch.Tensor, node_offsets: torch.Tensor,
                   rt_node_counts: torch.Tensor, codes: torch.Tensor, rt_prefixN: torch.Tensor,
                   rt_parents: torch.Tensor, min_coord: float, range: float, N: int,  # noqa: A002
                   status: torch.Tensor | None = None):
    """include/kernels/07_octree.hpp:5-14 (N = number of radix nodes)."""
    lib = _lib.load()
    m = oct_nodes.shape[0]
    ws = _workspace(lib.oct_octree_workspace_bytes(m), oct_nodes.device)
    _lib.check(lib.oct_make_oct_nodes(
        _ptr(oct_nodes, "oct_nodes", torch.int32), m,
        _ptr(node_offsets, "node_offsets", torch.int32, N),
        _ptr(rt_node_counts, "rt_node_counts", torch.int32, N),
        _ptr(codes, "codes", torch.int32, N + 1), _ptr(rt_prefixN, "rt_prefixN", torch.uint8, N),
        _ptr(rt_parents, "rt_parents", torch.int32, N), min_coord, range, N, _ptr(ws, "workspace"),
        ws.numel(), _ptr(status, "status"), _stream()), "k_MakeOctNodes")


# ------------------------------------------------------------------ stage 8 --
def k_LinkLeafNodes(nodes: torch.Tensor, node_offsets: torch.Tensor,
                    rt_node_counts: torch.Tensor, codes: torch.Tensor,
                    rt_hasLeafLeft: torch.Tensor, rt_hasLeafRight: torch.Tensor,
                    rt_prefixN: torch.Tensor, rt_parents: torch.Tensor,
                    rt_leftChild: torch.Tensor, N: int, status: torch.Tensor | None = None):
    """include/kernels/07_octree.hpp:16-25 (N = number of radix nodes)."""
    lib = _lib.load()
    m = nodes.shape[0]
    ws = _workspace(lib.oct_octree_workspace_bytes(m), nodes.device)
    _lib.check(lib.oct_link_leaf_nodes(
        _ptr(nodes, "nodes", torch.int32), m, _ptr(node_offsets, "node_offsets", torch.int32, N),
        _ptr(rt_node_counts, "rt_node_counts", torch.int32, N),
        _ptr(codes, "codes", torch.int32, N + 1),
        _ptr(rt_hasLeafLeft, "rt_hasLeafLeft", torch.uint8, N),
        _ptr(rt_hasLeafRight, "rt_hasLeafRight", torch.uint8, N),
        _ptr(rt_prefixN, "rt_prefixN", torch.uint8, N), _ptr(rt_parents, "rt_parents", torch.int32, N),
        _ptr(rt_leftChild, "rt_leftChild", torch.int32, N), N, _ptr(ws, "workspace"), ws.numel(),
        _ptr(status, "status"), _stream()), "k_LinkLeafNodes")


def k_InitDescending(sort: torch.Tensor, n: int) -> None:
    """include/kernels/00_init.hpp:5: sort[i] = n - i (uint32 in an int32
    CUDA tensor), on the current stream."""
    _lib.check(_lib.load().oct_init_descending(_ptr(sort, "sort", torch.int32, n), n, _stream()),
               "oct_init_descending")


def k_InitAscending(sort: torch.Tensor, n: int) -> None:
    """include/kernels/00_init.hpp:7: sort[i] = i, on the current stream."""
    _lib.check(_lib.load().oct_init_ascending(_ptr(sort, "sort", torch.int32, n), n, _stream()),
               "oct_init_ascending")


# ------------------------------------------------------------ consumers --
def k_InitRandomVec4_device(points: torch.Tensor, n: int, min_coord: float, rng: float,
                            seed: int) -> None:
    """gpu::k_InitRandomVec4 (kernels/cuda/00_init.cu:27-50) into a CUDA
    float32 [n, 4] tensor, on the current stream."""
    p = _ptr(points, "points", torch.float32, 4 * n)
    _lib.check(_lib.load().oct_init_random_vec4_device(p, n, min_coord, rng, seed, _stream()),
               "oct_init_random_vec4_device")


def morton_decode(codes: torch.Tensor, n: int, min_coord: float, rng: float) -> torch.Tensor:
    """morton32_to_xyz (include/shared/morton.h:45-80) of n codes: [n, 4] float32."""
    out = torch.empty((max(n, 1), 4), dtype=torch.float32, device=codes.device)
    _lib.check(_lib.load().oct_morton_decode(_ptr(codes, "codes", None, n), n, min_coord, rng,
                                             C.c_void_p(out.data_ptr()), _stream()),
               "oct_morton_decode")
    return out[:n]


def check_tree(nodes: torch.Tensor, n_nodes: int, codes: torch.Tensor, n_codes: int,
               root_prefix: int, root_code_len: int, root_index: int = 0) -> tuple:
    """checkTree (apps/cpu_demo/main.cpp:13-35) on the GPU: (visited,
    leaf checks, mismatches, rejected)."""
    lib = _lib.load()
    ws = _workspace(lib.oct_check_tree_workspace_bytes(n_nodes), nodes.device)
    counts = torch.zeros(4, dtype=torch.int64, device=nodes.device)
    _lib.check(lib.oct_check_tree(_ptr(nodes, "nodes", None, OCTNODE_WORDS * n_nodes), n_nodes,
                                  _ptr(codes, "codes", None, n_codes), n_codes,
                                  root_prefix & 0xFFFFFFFF,
                                  root_code_len, root_index, C.c_void_p(counts.data_ptr()),
                                  C.c_void_p(ws.data_ptr()), ws.numel(), _stream()),
               "oct_check_tree")
    return tuple(int(v) for v in counts.cpu().tolist())
