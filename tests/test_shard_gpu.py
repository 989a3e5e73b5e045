"""The batched build split over two ranks, each building its shard on the GPU.

Two processes (gloo for the host-side gather; both on cuda:0, whose kernels
never wait on each other) each build their clouds (ShardBuilder: the clouds
shard_clouds gives the rank, in one batched build) and all-gather per-cloud
hashes of every stage buffer. Together they must cover every cloud exactly once, and every cloud
must equal the oracle's build of it (apps/cpu_demo/main.cpp:72-154)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu

STAGES = ["sorted_unique", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent",
          "edge_count", "prefix_sum", "oct_nodes"]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _clouds():
    from pipeline_gb300 import datasets

    return datasets.batched(48, seed=13, lo=100, hi=60_000)


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch
    import torch.distributed as dist

    from oracle import oracle as O
    from pipeline_gb300.batch import ShardBuilder

    dist.init_process_group("gloo", rank=rank, world_size=world)
    clouds = _clouds()
    sizes = [len(c) for c in clouds]
    shard = ShardBuilder(sizes, rank, world, device="cuda:0")
    shard.build(clouds, [0.0] * len(sizes), [1024.0] * len(sizes))
    torch.cuda.synchronize()
    hashes = {}
    for c in shard.clouds:
        r = shard.cloud_result(c)
        hashes[c] = (r["n_unique"], r["n_oct"], r["status"],
                     [O.fnv1a64(np.asarray(r[k])) for k in STAGES])
    gathered = [None] * world
    dist.all_gather_object(gathered, hashes)
    if rank == 0:
        out.put(gathered)
    dist.destroy_process_group()


def test_two_ranks_build_their_shards_like_the_oracle():
    from oracle import oracle as O

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=600)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    clouds = _clouds()
    seen = {}
    for part in gathered:
        for c, h in part.items():
            assert c not in seen, c
            seen[c] = h
    assert sorted(seen) == list(range(len(clouds)))
    assert all(len(part) > 0 for part in gathered)
    for c, p in enumerate(clouds):
        want = O.build_all(p, 0.0, 1024.0)
        u, m, st, hs = seen[c]
        assert (u, st) == (want["n_unique"], 0), c
        if want["n_unique"] < 2:
            continue
        assert m == want["n_oct"], c
        assert hs == [O.fnv1a64(np.asarray(want[k])) for k in STAGES], c
