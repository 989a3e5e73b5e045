"""Multi-rank split of a batch (no collective on the data path): two gloo
ranks on CPU each take their clouds with shard_clouds and all-gather the
assignment; together they cover every cloud exactly once with balanced
point counts."""
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
