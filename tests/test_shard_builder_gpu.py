"""Sharded batched build in one process (ShardBuilder: one rank's share of a
batch split by shard_clouds). The ranks of 2-, 3- and 5-rank splits are built
one after another on one GPU (no rank waits on another: each is an independent batched
build), and together they must give every cloud of the batch exactly once,
each cloud equal to the oracle's build of it (apps/cpu_demo/main.cpp:72-154)
and to the same cloud of the whole batch built by one BatchOctreeBuilder;
the learned form likewise with one model shared by all ranks."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

STAGES = ["sorted_unique", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent",
          "edge_count", "prefix_sum", "oct_nodes"]


def _clouds(seed=4):
    from pipeline_gb300 import datasets

    rng = np.random.default_rng(seed)
    sizes = [0, 1, 2, 4096, 4097, 30000, 90000] + rng.integers(1, 20000, 17).tolist()
    clouds, mins, ranges = [], [], []
    for i, n in enumerate(sizes):
        if i % 3 == 0:
            p = rng.uniform(0, 1024, (n, 4))
        elif i % 3 == 1:
            p = datasets.gaussian_mixture(max(n, 1), 8, rng)[:n]
        else:
            p = rng.integers(0, 40, (n, 4)) * 1.0 + 0.25
        p = np.asarray(p, np.float32)
        p[:, 3] = 1
        shift = np.float32(-64.5 if i % 4 == 0 else 0.0)
        p[:, :3] += shift
        clouds.append(p)
        mins.append(float(shift))
        ranges.append(1024.0)
    return clouds, mins, ranges


def _same(got, want, c):
    assert got["n_unique"] == want["n_unique"], c
    if want["n_unique"] < 2:
        return
    assert (got["n_oct"], got["status"]) == (want["n_oct"], 0), c
    for key in STAGES:
        assert np.asarray(got[key]).tobytes() == np.asarray(want[key]).tobytes(), (c, key)


@pytest.fixture(scope="module")
def batch():
    from pipeline_gb300.batch import BatchOctreeBuilder

    clouds, mins, ranges = _clouds()
    sizes = [len(c) for c in clouds]
    whole = BatchOctreeBuilder(sizes)
    pts = torch.from_numpy(np.concatenate(clouds, 0)).cuda()
    mn = torch.tensor(mins, dtype=torch.float32, device="cuda")
    rg = torch.tensor(ranges, dtype=torch.float32, device="cuda")
    whole.build(pts, mn, rg)
    counts = whole.cloud_counts()
    ref = [whole.cloud_result(c, counts) for c in range(len(clouds))]
    return clouds, mins, ranges, pts, mn, rg, ref


@pytest.mark.parametrize("world", [2, 3, 5])
def test_shards_together_equal_the_whole_batch_and_the_oracle(batch, world):
    from pipeline_gb300.batch import ShardBuilder

    clouds, mins, ranges, pts, mn, rg, ref = batch
    sizes = [len(c) for c in clouds]
    seen = []
    for rank in range(world):
        sb = ShardBuilder(sizes, rank, world)
        # whole-batch inputs on the device: the rank packs its own rows
        sb.build(pts, mn, rg)
        for c in sb.clouds:
            got = sb.cloud_result(c)
            _same(got, ref[c], c)
            _same(got, O.build_all(clouds[c], mins[c], ranges[c]), c)
        assert set(sb.cloud_counts()) == set(sb.clouds)
        seen += sb.clouds
    assert sorted(seen) == list(range(len(clouds)))


def test_shard_from_host_clouds_and_its_graph_replay(batch):
    """Per-cloud host arrays as input (what a rank reads from its own files),
    captured once and replayed: the same results as the whole batch."""
    from pipeline_gb300.batch import ShardBuilder

    clouds, mins, ranges, _, _, _, ref = batch
    sizes = [len(c) for c in clouds]
    sb = ShardBuilder(sizes, 1, 2)
    sb.capture(clouds, mins, ranges)
    for _ in range(2):
        sb.replay()
    torch.cuda.synchronize()
    for c in sb.clouds:
        _same(sb.cloud_result(c), ref[c], c)
    with pytest.raises(ValueError):
        sb.cloud_result(next(c for c in range(len(clouds)) if c not in sb.clouds))


def test_learned_shards_match_the_oracle():
    """Scan-like frames split over two ranks, both ranks' learned batched
    builds driven by one model fit on the first frames."""
    from pipeline_gb300 import datasets
    from pipeline_gb300.batch import ShardBuilder
    from pipeline_gb300.kernels import k_ComputeMortonCode
    from pipeline_gb300.learned import LearnedCDF

    fr, mins, ranges = datasets.scan_frames(24, seed=9)
    codes = []
    for f, a, r in zip(fr[:6], mins[:6], ranges[:6]):
        k = torch.empty(len(f), dtype=torch.int32, device="cuda")
        k_ComputeMortonCode(torch.from_numpy(np.ascontiguousarray(f)).cuda(), k, len(f), a, r)
        codes.append(k)
    model = LearnedCDF(max_segments=1024).fit(torch.cat(codes), n_segments=1024, steps=100,
                                              lr=0.05, n_buckets=64)
    test, tmins, tranges = fr[6:], mins[6:], ranges[6:]
    sizes = [len(f) for f in test]
    seen = []
    for rank in range(2):
        sb = ShardBuilder(sizes, rank, 2, model=model, n_buckets=64)
        sb.build(test, tmins, tranges)
        for c in sb.clouds:
            _same(sb.cloud_result(c), O.build_all(test[c], tmins[c], tranges[c]), c)
        seen += sb.clouds
    assert sorted(seen) == list(range(len(test)))
