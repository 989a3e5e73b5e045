"""Whole-build octree stage (octree_tiled.cu) under every tiling.

The whole build makes its octree slots per tile of radix nodes in shared
memory and rebuilds the slots that receive writes from other tiles in a
fix-up pass. Small tiles and chunks push most of the work through the fix-up
pass and the chunk loop; every tiling must give the oracle's bytes (the
reference's sequential stages 7-8, include/shared/oct.h:9-134)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from pipeline_gb300 import _lib

STAGES = ["sorted_unique", "prefix_n", "left_child", "parent", "edge_count", "prefix_sum",
          "oct_nodes"]
TILINGS = [(512, 512), (512, 16), (96, 512), (32, 8), (7, 3), (1, 1)]


def _clouds():
    from pipeline_gb300 import datasets

    return [("uniform_50k", O.init_random_vec4(50_000, seed=21), 0.0, 1024.0),
            ("box_30k", O.init_random_vec4(30_000, 500.0, 24.0, 22), 0.0, 1024.0),
            ("clustered_60k", datasets.clustered(60_000, seed=23), 0.0, 1024.0),
            ("tiny_40", O.init_random_vec4(40, seed=24), 0.0, 1024.0),
            ("shifted_20k", O.init_random_vec4(20_000, -7.5, 3.25, 25), -7.5, 3.25)]


@pytest.mark.gpu
@pytest.mark.parametrize("tiling", TILINGS)
def test_every_tiling_matches_oracle(tiling):
    from pipeline_gb300.pipeline import OctreeBuilder

    lib = _lib.load()
    assert lib.oct_set_octree_tiling(*tiling) == _lib.OCT_OK
    try:
        for name, pts, mn, rg in _clouds():
            b = OctreeBuilder(len(pts))
            b.build(torch.from_numpy(pts).cuda(), mn, rg)
            got, want = b.result(), O.build_all(pts, mn, rg)
            assert (got["n_unique"], got["n_oct"], got["status"]) == (
                want["n_unique"], want["n_oct"], 0), name
            for key in STAGES:
                assert np.asarray(got[key]).tobytes() == np.asarray(want[key]).tobytes(), (name, key)
    finally:
        lib.oct_set_octree_tiling(0, 0)


@pytest.mark.parametrize("tiling", TILINGS)
def test_tilings_used_above_are_accepted(tiling):
    lib = _lib.load()
    try:
        assert lib.oct_set_octree_tiling(*tiling) == _lib.OCT_OK
    finally:
        lib.oct_set_octree_tiling(0, 0)


def test_tiling_rejects_out_of_range_values():
    lib = _lib.load()
    for bad in [(0, 5), (5, 0), (513, 8), (8, 513), (-1, -1)]:
        assert lib.oct_set_octree_tiling(*bad) == _lib.OCT_ERR_INVALID_ARG
    assert lib.oct_set_octree_tiling(0, 0) == _lib.OCT_OK
