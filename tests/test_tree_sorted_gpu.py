"""GPU parity of the delta-based radix tree (oct_build_radix_tree_sorted, the
form the whole-cloud builds use) against the per-node search stage
(k_BuildRadixTree), the oracle and the reference-generated fixtures.

Code sets cover tile edges (4,096 positions), runs of consecutive codes,
clusters, and both root forms: the reference's node 0 spans [0, n - 1], so
when the smallest adjacent delta sits at n - 1 the root is "short".
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TREE = ["prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent"]


def K():
    from pipeline_gb300 import kernels

    return kernels


def _garbage(n, dtype):
    if dtype == torch.uint8:
        return torch.full((max(n, 1),), 0x5A, dtype=torch.uint8, device="cuda")
    return torch.full((max(n, 1),), 0x5A5A5A5A, dtype=torch.int32, device="cuda")


def _outputs(n):
    return dict(prefix_n=_garbage(n, torch.uint8), has_leaf_left=_garbage(n, torch.uint8),
                has_leaf_right=_garbage(n, torch.uint8), left_child=_garbage(n, torch.int32),
                parent=_garbage(n, torch.int32))


def sorted_tree(codes: np.ndarray):
    n = len(codes) - 1
    c = torch.from_numpy(np.ascontiguousarray(codes, np.uint32).view(np.int32)).cuda()
    out = _outputs(n)
    ec = _garbage(n, torch.int32)
    K().build_radix_tree_sorted(n, c, out["prefix_n"], out["has_leaf_left"],
                                out["has_leaf_right"], out["left_child"], out["parent"], ec)
    torch.cuda.synchronize()
    got = {k: v[:n].cpu().numpy() for k, v in out.items()}
    return got, ec[:n].cpu().numpy()


def search_tree(codes: np.ndarray):
    n = len(codes) - 1
    c = torch.from_numpy(np.ascontiguousarray(codes, np.uint32).view(np.int32)).cuda()
    out = _outputs(n)
    K().k_BuildRadixTree(n, c, out["prefix_n"], out["has_leaf_left"], out["has_leaf_right"],
                         out["left_child"], out["parent"])
    torch.cuda.synchronize()
    return {k: v[:n].cpu().numpy() for k, v in out.items()}


def code_set(kind: str, n_codes: int, rng) -> np.ndarray:
    if kind == "uniform":
        c = np.unique(rng.integers(0, 1 << 30, n_codes + n_codes // 8 + 16))
        c = rng.permutation(c)[:n_codes]
    elif kind == "consecutive":
        start = int(rng.integers(0, (1 << 30) - n_codes))
        c = np.arange(start, start + n_codes)
    elif kind == "clustered":
        centres = rng.integers(0, 1 << 30, 7)
        span = 2 * n_codes // 7 + 64  # dense enough to hold n_codes between them
        parts = [(ctr + rng.integers(0, max(1 << int(rng.integers(8, 20)), span), n_codes))
                 % (1 << 30) for ctr in centres]
        c = rng.permutation(np.unique(np.concatenate(parts)))[:n_codes]
    elif kind == "short_root":  # the smallest delta at n - 1: one code far above the rest
        c = np.unique(rng.integers(0, 1 << 26, n_codes + n_codes // 4 + 16))
        c = np.append(rng.permutation(c)[:n_codes - 1], (1 << 29) + 12345)
    elif kind == "low_outlier":  # the smallest delta at 0
        c = np.unique(rng.integers(1 << 29, (1 << 29) + (1 << 24), n_codes + n_codes // 4 + 16))
        c = np.append(rng.permutation(c)[:n_codes - 1], 7)
    elif kind == "two_high":  # the smallest delta at n - 2 (right end of node 0 is a leaf pair)
        c = np.unique(rng.integers(0, 1 << 24, n_codes + n_codes // 4 + 16))
        c = np.append(rng.permutation(c)[:n_codes - 2], [(1 << 29) + 1, (1 << 29) + 2])
    else:
        raise ValueError(kind)
    c = np.unique(np.asarray(c, np.int64)).astype(np.uint32)
    assert len(c) == n_codes, (kind, n_codes, len(c))
    return c


def _same(got, ref, label):
    for k in TREE:
        r = np.asarray(ref[k])
        g = np.asarray(got[k]).astype(r.dtype)
        if not np.array_equal(g, r):
            bad = np.nonzero(g != r)[0]
            raise AssertionError(f"{label} {k}: {len(bad)} differ, first {bad[:4]}: "
                                 f"got {g[bad[:4]]} want {r[bad[:4]]}")


def test_small_cases_match_fixtures(small_cases):
    for name, case in small_cases.items():
        codes = case["sorted_unique"]
        got, ec = sorted_tree(codes)
        _same(got, case, name)
        assert ec.tobytes() == case["edge_count"].tobytes(), name


@pytest.mark.parametrize("n_codes", [2, 3, 4, 5, 17, 33, 64, 65, 4095, 4096, 4097, 4098,
                                     8192, 8193, 12289, 20000])
@pytest.mark.parametrize("kind", ["uniform", "consecutive", "clustered", "short_root",
                                  "low_outlier", "two_high"])
def test_matches_oracle(kind, n_codes):
    rng = np.random.default_rng(n_codes * 7 + len(kind))
    codes = code_set(kind, n_codes, rng)
    n = n_codes - 1
    ref = O.build_radix_tree(codes, n)
    got, ec = sorted_tree(codes)
    _same(got, ref, f"{kind}/{n_codes}")
    assert np.array_equal(ec, O.edge_count(ref["prefix_n"], ref["parent"])), (kind, n_codes)


@pytest.mark.parametrize("kind,n_codes", [("uniform", (1 << 20) + 3), ("clustered", 1 << 20),
                                          ("consecutive", (1 << 21) + 1),
                                          ("short_root", 3 * 4096 * 512 + 77)])
def test_large_matches_search_stage(kind, n_codes):
    """Past one 512-tile block of the cross-tile scan; the per-node search
    stage (itself checked against the oracle) is the reference here."""
    rng = np.random.default_rng(n_codes)
    codes = code_set(kind, n_codes, rng)
    got, ec = sorted_tree(codes)
    ref = search_tree(codes)
    _same(got, ref, f"{kind}/{n_codes}")
    assert np.array_equal(ec, O.edge_count(ref["prefix_n"], ref["parent"]))


def test_one_node():
    codes = np.array([5, 9], np.uint32)
    got, ec = sorted_tree(codes)
    _same(got, O.build_radix_tree(codes, 1), "n=1")
    assert ec.tolist() == [0]
