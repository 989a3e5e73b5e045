"""Failure detection without a GPU fault: bounded waits and walks.

The reference's look-back spins (kernels/cuda/02_sort.cu:461-479) and its
LinkLeaf parent walk (include/shared/oct.h:111-113) have no bound. Here every
look-back wait gives up after a time bound and every walk after a step bound;
both set a status bit the host reads, and the kernel returns with all its
accesses in bounds, so the context stays usable. These tests make a wait run
out (a predecessor flag that nothing publishes, with a short bound) and a
walk run out (a parent cycle), and check the status bits and that the next
build is still correct.
"""
import ctypes as C
import time

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pipeline_gb300 import _lib

pytestmark = pytest.mark.gpu


def _clean_build_still_matches_oracle():
    from pipeline_gb300.pipeline import OctreeBuilder

    pts = O.init_random_vec4(20_000, seed=5)
    b = OctreeBuilder(len(pts))
    b.build(torch.from_numpy(pts).cuda(), 0.0, 1024.0)
    got, want = b.result(), O.build_all(pts, 0.0, 1024.0)
    assert got["status"] == 0
    assert got["oct_nodes"].tobytes() == want["oct_nodes"].tobytes()


@pytest.mark.parametrize("which", [_lib.OCT_DIAG_WAIT_SORT, _lib.OCT_DIAG_WAIT_SCAN],
                         ids=["sort_digit_lookback", "scan_warp_lookback"])
def test_lookback_wait_gives_up_within_its_bound(which):
    lib = _lib.load()
    ws = torch.empty(max(lib.oct_diag_wait_workspace_bytes(), 256), dtype=torch.uint8, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    limit_ns = 2_000_000  # 2 ms
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc = lib.oct_diag_lookback_timeout(which, limit_ns, C.c_void_p(ws.data_ptr()), ws.numel(),
                                       C.c_void_p(status.data_ptr()), s)
    _lib.check(rc, "oct_diag_lookback_timeout")
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    assert int(status.item()) & _lib.OCT_STATUS_SPIN_TIMEOUT
    assert elapsed < 0.5, elapsed  # 2 ms bound plus launch and copy overheads
    # the tile that gave up still published its word (nothing waits forever on it)
    if which == _lib.OCT_DIAG_WAIT_SORT:
        words = ws[:8192].view(torch.int32).cpu().numpy().view(np.uint32)
        assert words[1024] >> 30 == 2
    else:
        words = ws[:16].view(torch.int64).cpu().numpy().view(np.uint64)
        assert int(words[1]) >> 62 == 2
    _clean_build_still_matches_oracle()


def test_diag_rejects_unbounded_or_bad_arguments():
    lib = _lib.load()
    ws = torch.empty(8192, dtype=torch.uint8, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    p, st = C.c_void_p(ws.data_ptr()), C.c_void_p(status.data_ptr())
    assert lib.oct_diag_lookback_timeout(0, 0, p, 8192, st, None) == _lib.OCT_ERR_INVALID_ARG
    assert lib.oct_diag_lookback_timeout(0, 2_000_000_000, p, 8192, st, None) == _lib.OCT_ERR_INVALID_ARG
    assert lib.oct_diag_lookback_timeout(7, 1000, p, 8192, st, None) == _lib.OCT_ERR_INVALID_ARG
    assert lib.oct_diag_lookback_timeout(0, 1000, p, 100, st, None) == _lib.OCT_ERR_WORKSPACE


def _tree_arrays(parent, counts, hll, hlr, left):
    n = len(parent)
    d = lambda a, t: torch.tensor(a, dtype=t, device="cuda")  # noqa: E731
    codes = d(np.arange(n + 1, dtype=np.int32) * 8, torch.int32)
    return dict(offsets=d(np.zeros(n, np.int32), torch.int32), counts=d(counts, torch.int32),
                codes=codes, hll=d(hll, torch.uint8), hlr=d(hlr, torch.uint8),
                prefix=d(np.full(n, 27, np.uint8), torch.uint8), parent=d(parent, torch.int32),
                left=d(left, torch.int32))


def test_link_walk_on_a_parent_cycle_sets_walk_limit():
    from pipeline_gb300.kernels import empty_oct_nodes, k_LinkLeafNodes

    # nodes 1 and 2 are each other's parent and own no octree node: the
    # reference's walk (while counts[rt_node] == 0) would never end
    a = _tree_arrays(parent=[0, 2, 1, 2], counts=[0, 0, 0, 0], hll=[0, 1, 0, 0],
                     hlr=[0, 0, 0, 0], left=[0, 1, 0, 0])
    nodes = empty_oct_nodes(1)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    k_LinkLeafNodes(nodes, a["offsets"], a["counts"], a["codes"], a["hll"], a["hlr"], a["prefix"],
                    a["parent"], a["left"], 4, status)
    torch.cuda.synchronize()
    assert int(status.item()) & _lib.OCT_STATUS_WALK_LIMIT
    _clean_build_still_matches_oracle()


def test_make_walk_with_parent_out_of_range_sets_walk_limit():
    from pipeline_gb300.kernels import empty_oct_nodes, k_MakeOctNodes

    a = _tree_arrays(parent=[0, 77, 0, 0], counts=[0, 1, 0, 0], hll=[0] * 4, hlr=[0] * 4,
                     left=[0] * 4)
    a["offsets"] = torch.tensor([0, 1, 1, 1], dtype=torch.int32, device="cuda")
    nodes = empty_oct_nodes(2)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    k_MakeOctNodes(nodes, a["offsets"], a["counts"], a["codes"], a["prefix"], a["parent"], 0.0,
                   1024.0, 4, status)
    torch.cuda.synchronize()
    assert int(status.item()) & _lib.OCT_STATUS_WALK_LIMIT
