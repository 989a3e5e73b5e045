"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
symbol include/*.h declares. Only host-side entry points are called here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from pipeline_gb300 import _lib
from pipeline_gb300 import build as B

HEADERS = [os.path.join(B.INCLUDE, f) for f in os.listdir(B.INCLUDE) if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        names.update(re.findall(r"^OCT_API\s+[\w\s\*]+?\b(oct_\w+)\s*\(", text, re.M))
    return names


def test_library_builds_and_loads():
    path = B.build()
    assert os.path.exists(path)
    lib = _lib.load()
    assert lib.oct_built_arch() == 1033
    assert lib.oct_version() >= 100


def test_every_declared_symbol_is_exported():
    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 20
    for name in sorted(names):
        assert hasattr(lib, name), name
    # ...and the Python binding declares a signature for each one.
    assert names == set(_lib.SIGNATURES), names ^ set(_lib.SIGNATURES)


def test_workspace_sizes_are_host_computable():
    lib = _lib.load()
    assert lib.oct_sort_workspace_bytes(1 << 24, 30) > 0
    assert lib.oct_sort_workspace_bytes(-1, 30) == 0
    assert lib.oct_sort_workspace_bytes(10, 33) == 0
    assert lib.oct_unique_workspace_bytes(1 << 20) % 256 == 0
    a = lib.oct_build_workspace_bytes(1 << 20, 1 << 20)
    b = lib.oct_build_workspace_bytes(1 << 21, 1 << 20)
    assert 0 < a < b
    # 30-bit Morton keys take 3 passes of 10-bit digits: histogram + look-back
    # control stays a small fraction of the keys themselves.
    n = 1 << 24
    assert lib.oct_sort_workspace_bytes(n, 30) < 4 * n


@pytest.mark.parametrize("n,nb", [(1000, 4096), (1 << 20, 1024), (1 << 24, 4096), (1 << 24, 256)])
def test_learned_workspace_holds_every_bucket_range(n, nb):
    """The learned sort bins keys into one fixed range per bucket: at least
    4 B x nb x max(16,384, 2 n / nb) keys (rounded to whole 128-byte lines)."""
    lib = _lib.load()
    mean = -(-n // nb)
    cap = -(-max(16384, 2 * mean) // 32) * 32
    ws = lib.oct_lsort_workspace_bytes(n, nb, 4096)
    assert ws >= 4 * nb * cap
    assert ws < 4 * nb * cap + 16 * n + (64 << 20)  # the rest: keys, fallback sort, tables
    assert lib.oct_build_learned_workspace_bytes(n, n, nb, 4096) > ws
    assert lib.oct_lsort_workspace_bytes(n, 1 << 20, 4096) == 0  # bucket tables past shared memory


def test_invalid_arguments_rejected_before_any_device_work():
    lib = _lib.load()
    assert lib.oct_morton_encode(None, None, -1, 0.0, 1.0, None, None) == _lib.OCT_ERR_INVALID_ARG
    assert lib.oct_sort_keys(None, None, -5, 30, None, 0, None, None) == _lib.OCT_ERR_INVALID_ARG
    assert lib.oct_sort_keys(None, None, 10, 40, None, 0, None, None) == _lib.OCT_ERR_INVALID_ARG
    assert lib.oct_build_octree(None, 10, 0.0, 1.0, None, None, 0, None) == _lib.OCT_ERR_INVALID_ARG
    assert lib.oct_build_radix_tree(-1, None, None, None, None, None, None, None) == _lib.OCT_ERR_INVALID_ARG
    # misaligned workspace
    fake = C.c_void_p(0x1000 + 8)
    assert lib.oct_unique(fake, 100, fake, fake, 1 << 20, None, None) == _lib.OCT_ERR_INVALID_ARG
    # too-small workspace (256-aligned fake pointers; rejected before use)
    al = C.c_void_p(0x100000)
    assert lib.oct_unique(al, 100, al, al, 8, None, None) == _lib.OCT_ERR_WORKSPACE


def test_octree_node_limit_rejected_before_any_device_work():
    """Octree write tags hold the radix-node index in 27 bits: larger octree
    stages and whole builds with an octree answer OCT_ERR_TOO_LARGE."""
    lib = _lib.load()
    big = (1 << 27) - 1 + 1
    assert lib.oct_make_oct_nodes(None, 10, None, None, None, None, None, 0.0, 1.0, big, None, 0,
                                  None, None) == _lib.OCT_ERR_TOO_LARGE
    out = _lib.OctBuildOutputs()
    out.nodes_capacity = 1
    out.d_counts = C.c_void_p(0x100000)
    assert lib.oct_build_octree(None, big + 1, 0.0, 1.0, C.byref(out), None, 0, None) == \
        _lib.OCT_ERR_TOO_LARGE
    sizes = (C.c_int32 * 2)(1000, big + 1)
    assert not lib.oct_batch_plan_create(2, sizes, None)


def test_host_generator_matches_reference(golden):
    """oct_init_random_vec4 reproduces k_InitRandomVec4's points."""
    from pipeline_gb300.kernels import k_InitRandomVec4

    pts = k_InitRandomVec4(None, 4, 0.0, 1024.0, 114514)
    assert pts.tolist() == golden["cfg1_uniform_1m"]["first_points"]


def test_host_generator_hash(golden):
    from oracle import oracle as O
    from pipeline_gb300.kernels import k_InitRandomVec4

    g = golden["cfg1_uniform_1m"]
    pts = k_InitRandomVec4(None, g["n"], g["min"], g["range"], g["seed"])
    assert O.fnv1a64(pts) == g["input_hash"]
