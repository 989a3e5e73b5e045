"""GPU parity of the whole build's two forms of stages 2-3 on clouds large
enough (2^22+ points) for the MSD form to be considered: the device takes the
MSD form (top-digit scatter, per-bucket bitmaps, pack) for even clouds and
falls back to the LSD radix passes for uneven ones; both must give the
oracle's bytes for every stage output."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

STAGES = ["sorted_unique", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent",
          "edge_count", "prefix_sum", "oct_nodes"]
MIN_N = 1 << 22


def _build(pts):
    from pipeline_gb300.pipeline import OctreeBuilder

    n = len(pts)
    b = OctreeBuilder(n)
    b.build(torch.from_numpy(np.ascontiguousarray(pts)).cuda(), 0.0, 1024.0)
    return b.result(), b.sort_form()


def _check(pts, form, label):
    res, got_form = _build(pts)
    assert got_form == form, (label, got_form)
    expect = O.build_all(pts, 0.0, 1024.0)
    assert (res["n_unique"], res["n_oct"], res["status"]) == \
        (expect["n_unique"], expect["n_oct"], 0), label
    for key in STAGES:
        assert res[key].tobytes() == np.asarray(expect[key]).tobytes(), (label, key)


def test_msd_form_even_cloud_with_duplicates():
    # points on a 1/4-unit grid: many cells hold several points (duplicate codes)
    rng = np.random.default_rng(5)
    n = MIN_N + 12345
    pts = np.ones((n, 4), np.float32)
    pts[:, :3] = np.floor(rng.uniform(0, 1024, (n, 3)) * 4) / 4
    _check(pts, 1, "grid")


def test_msd_form_heavy_duplicates():
    # 64^3 cell centres: every bucket holds ~4,000 keys but only ~256 codes
    rng = np.random.default_rng(6)
    n = MIN_N + 4321
    pts = np.ones((n, 4), np.float32)
    pts[:, :3] = (rng.integers(0, 64, (n, 3)) * 16 + 8).astype(np.float32)
    _check(pts, 1, "coarse grid")


def test_msd_form_with_empty_buckets():
    # x in the lower half of the box: the top-digit buckets of the upper half
    # stay empty, the others hold twice the mean
    rng = np.random.default_rng(8)
    n = MIN_N + 99
    pts = np.ones((n, 4), np.float32)
    pts[:, 0] = rng.uniform(0, 512, n)
    pts[:, 1:3] = rng.uniform(0, 1024, (n, 2))
    _check(pts, 1, "half box")


def test_msd_form_even_cloud():
    n = MIN_N + 1
    _check(O.init_random_vec4(n, 0.0, 1024.0, seed=77), 1, "uniform")


def test_lsd_fallback_for_uneven_cloud():
    rng = np.random.default_rng(9)
    n = MIN_N + 777
    c = rng.uniform(100, 900, (6, 3))
    idx = rng.integers(0, 6, n)
    pts = np.ones((n, 4), np.float32)
    pts[:, :3] = np.clip(rng.normal(c[idx], 12.0), 0, np.nextafter(np.float32(1024), 0))
    _check(pts, 2, "clusters")


def test_below_msd_size_uses_lsd():
    n = MIN_N - 1
    _check(O.init_random_vec4(n, 0.0, 1024.0, seed=3), 0, "below")


def test_captured_build_takes_either_form():
    # One captured graph, replayed over an even cloud (MSD branch) and then,
    # with the points changed in place, over a clustered one (LSD branch) and
    # back: the branch is chosen on the device at every replay.
    from pipeline_gb300.pipeline import OctreeBuilder

    n = MIN_N + 333
    even = O.init_random_vec4(n, 0.0, 1024.0, seed=21)
    rng = np.random.default_rng(22)
    c = rng.uniform(100, 900, (5, 3))
    idx = rng.integers(0, 5, n)
    clustered = np.ones((n, 4), np.float32)
    clustered[:, :3] = np.clip(rng.normal(c[idx], 10.0), 0, np.nextafter(np.float32(1024), 0))
    d_pts = torch.from_numpy(np.ascontiguousarray(even)).cuda()
    b = OctreeBuilder(n)
    b.capture(d_pts, 0.0, 1024.0)
    for pts, form in ((even, 1), (clustered, 2), (even, 1)):
        d_pts.copy_(torch.from_numpy(np.ascontiguousarray(pts)))
        b.nodes.fill_(-1)
        b.replay()
        res = b.result()
        assert b.sort_form() == form
        expect = O.build_all(pts, 0.0, 1024.0)
        assert (res["n_unique"], res["n_oct"], res["status"]) == \
            (expect["n_unique"], expect["n_oct"], 0), form
        for key in STAGES:
            assert res[key].tobytes() == np.asarray(expect[key]).tobytes(), (form, key)
