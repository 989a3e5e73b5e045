"""Multi-rank split of a batch (no collective on the data path): two gloo
ranks on CPU each take their clouds with shard_clouds and all-gather the
assignment; together they cover every cloud exactly once with balanced
point counts, and each rank's packed input (pack_shard, which ShardBuilder
uses to feed its batched build) holds exactly its clouds' rows, mins and
ranges."""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, sizes, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from pipeline_gb300.batch import shard_clouds

    mine = shard_clouds(sizes, world)[rank]
    mask = torch.zeros(len(sizes), dtype=torch.int32)
    mask[mine] = 1
    gathered = [torch.zeros_like(mask) for _ in range(world)]
    dist.all_gather(gathered, mask)
    if rank == 0:
        out.put([g.tolist() for g in gathered])
    dist.destroy_process_group()


def test_two_rank_shard_covers_each_cloud_once():
    rng = np.random.default_rng(0)
    sizes = np.exp(rng.uniform(np.log(1000), np.log(1_000_000), 512)).astype(int).tolist()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    masks = np.array(q.get(timeout=120))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert np.all(masks.sum(0) == 1)
    loads = masks @ np.array(sizes)
    assert abs(loads[0] - loads[1]) <= max(sizes)


def test_shard_is_deterministic_and_balanced():
    from pipeline_gb300.batch import shard_clouds

    sizes = [5, 9, 1, 7, 7, 3]
    a = shard_clouds(sizes, 3)
    assert a == shard_clouds(sizes, 3)
    assert sorted(sum(a, [])) == list(range(6))
    loads = [sum(sizes[c] for c in s) for s in a]
    assert max(loads) - min(loads) <= max(sizes)


def _batch(sizes):
    """Whole-batch points whose x is the row's index in the batch, per-cloud
    mins and ranges that name their cloud."""
    n = int(sum(sizes))
    pts = torch.zeros((n, 4), dtype=torch.float32)
    pts[:, 0] = torch.arange(n, dtype=torch.float32)
    pts[:, 3] = 1
    c = torch.arange(len(sizes), dtype=torch.float32)
    return pts, -0.5 * c, 1024.0 + c


def _pack_worker(rank, world, port, sizes, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from pipeline_gb300.batch import pack_shard, shard_clouds, shard_slices

    pts, mins, ranges = _batch(sizes)
    mine = shard_clouds(sizes, world)[rank]
    p, m, r = pack_shard(pts, mins, ranges, sizes, mine)
    # the list-of-clouds form packs the same rows
    per_cloud = [pts[lo:hi].numpy() for lo, hi in shard_slices(sizes, range(len(sizes)))]
    p2, m2, r2 = pack_shard(per_cloud, mins.tolist(), ranges.tolist(), sizes, mine)
    same = bool(torch.equal(p, p2) and torch.equal(m, m2) and torch.equal(r, r2))
    got = {}
    off = 0
    for k, c in enumerate(mine):
        rows = p[off:off + sizes[c], 0].to(torch.int64)
        off += sizes[c]
        got[c] = (int(rows[0]) if len(rows) else -1, len(rows),
                  bool(torch.equal(rows, torch.arange(int(rows[0]), int(rows[0]) + len(rows)))
                       if len(rows) else True),
                  float(m[k]), float(r[k]))
    gathered = [None] * world
    dist.all_gather_object(gathered, {"rows": got, "total": off == p.shape[0], "same": same})
    if rank == 0:
        out.put(gathered)
    dist.destroy_process_group()


def test_two_rank_packed_shards_hold_exactly_their_clouds():
    rng = np.random.default_rng(3)
    sizes = [0, 1, 4096, 4097] + rng.integers(0, 3000, 40).tolist()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_pack_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    ranks = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    start = np.concatenate([[0], np.cumsum(sizes)])
    seen = {}
    for rk in ranks:
        assert rk["total"] and rk["same"]
        for c, v in rk["rows"].items():
            assert c not in seen
            seen[c] = v
    assert sorted(seen) == list(range(len(sizes)))
    for c, (first, count, contiguous, mn, rg) in seen.items():
        assert count == sizes[c] and contiguous
        assert first == (start[c] if sizes[c] else -1)
        assert (mn, rg) == (-0.5 * c, 1024.0 + c)


def test_shard_slices_tile_the_batch():
    from pipeline_gb300.batch import shard_clouds, shard_slices

    sizes = [3, 0, 7, 1, 0, 12]
    for world in (1, 2, 4, 8):
        rows = []
        for mine in shard_clouds(sizes, world):
            for lo, hi in shard_slices(sizes, mine):
                rows.extend(range(lo, hi))
        assert sorted(rows) == list(range(sum(sizes)))


def test_rank_without_clouds_builds_nothing():
    """More ranks than clouds: the extra rank plans no build and touches no
    device; ranks outside [0, world) are rejected."""
    import pytest

    from pipeline_gb300.batch import ShardBuilder

    sb = ShardBuilder([5, 7], 2, 3, device="cpu")
    assert sb.clouds == [] and sb.builder is None and sb.cloud_counts() == {}
    sb.build([np.zeros((5, 4), np.float32), np.zeros((7, 4), np.float32)], [0.0, 0.0],
             [1.0, 1.0])
    sb.replay()
    assert sb.capture([np.zeros((5, 4), np.float32)] * 2, [0.0] * 2, [1.0] * 2) is None
    with pytest.raises(ValueError):
        ShardBuilder([5, 7], 3, 3, device="cpu")
    with pytest.raises(ValueError):
        ShardBuilder([5, 7], 0, 0, device="cpu")


def test_pack_shard_rejects_points_that_do_not_match_the_sizes():
    import pytest

    from pipeline_gb300.batch import pack_shard

    sizes = [3, 2]
    good = [np.zeros((3, 4), np.float32), np.ones((2, 4), np.float32)]
    pts, mn, rg = pack_shard(good, [0.0, 1.0], [8.0, 9.0], sizes, [1])
    assert pts.shape == (2, 4) and float(pts.sum()) == 8.0
    assert mn.tolist() == [1.0] and rg.tolist() == [9.0]
    with pytest.raises(ValueError):
        pack_shard([good[0], np.ones((3, 4), np.float32)], [0.0, 1.0], [8.0, 9.0], sizes, [1])
    with pytest.raises(ValueError):
        pack_shard(good[:1], [0.0], [8.0], sizes, [0])
    with pytest.raises(ValueError):
        pack_shard(torch.zeros((4, 4)), [0.0, 1.0], [8.0, 9.0], sizes, [0])
    with pytest.raises(ValueError):
        pack_shard(torch.zeros((5, 3)), [0.0, 1.0], [8.0, 9.0], sizes, [0])
    whole = np.arange(20, dtype=np.float32).reshape(5, 4)  # a numpy batch packs like a tensor
    pts, _, _ = pack_shard(whole, [0.0, 1.0], [8.0, 9.0], sizes, [1, 0])
    assert pts[:, 0].tolist() == [12.0, 16.0, 0.0, 4.0, 8.0]
