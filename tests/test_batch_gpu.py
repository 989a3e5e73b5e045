"""Batched build: every cloud bit-exact with the oracle (and so with the
single-cloud path), including degenerate clouds and clouds that hit the O7
walk; CUDA-graph replays deterministic."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

STAGES = ["sorted_unique", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent",
          "edge_count", "prefix_sum", "oct_nodes"]


def mixed_clouds(seed=0):
    from pipeline_gb300 import datasets

    rng = np.random.default_rng(seed)
    clouds, mins, ranges = [], [], []
    specs = [0, 1, 2, 3, 5, 17, 100, 1000, 4095, 4096, 4097, 8191, 8192, 8193, 12289, 30000, 70000,
             150000]
    for i, n in enumerate(specs + list(rng.integers(1, 20000, 22))):
        kind = i % 4
        if kind == 0:
            p = rng.uniform(0, 1024, (n, 4))
        elif kind == 1:
            p = datasets.gaussian_mixture(max(n, 1), 8, rng)[:n]
        elif kind == 2:
            p = rng.uniform(0, 30, (n, 4))
            if n:
                p[0, :3] = 1023.0
        else:
            p = rng.integers(0, 12, (n, 4)) * 1.0 + 0.5
        p = np.asarray(p, np.float32)
        p[:, 3] = 1
        # per-cloud quantisation: some clouds use a shifted frame
        if i % 5 == 0 and n:
            shift = np.float32(-100.25)
            p[:, :3] += shift
            mins.append(float(shift))
            ranges.append(1024.0)
        else:
            mins.append(0.0)
            ranges.append(1024.0)
        clouds.append(p)
    return clouds, mins, ranges


def build_batch(clouds, mins, ranges):
    from pipeline_gb300.batch import BatchOctreeBuilder

    sizes = [len(c) for c in clouds]
    b = BatchOctreeBuilder(sizes)
    pts = torch.from_numpy(np.concatenate(clouds, 0) if sum(sizes) else np.zeros((1, 4), np.float32)).cuda()
    mn = torch.tensor(mins, dtype=torch.float32, device="cuda")
    rg = torch.tensor(ranges, dtype=torch.float32, device="cuda")
    return b, pts, mn, rg


def check_cloud(b, counts, c, pts, mn, rg):
    res = b.cloud_result(c, counts)
    want = O.build_all(pts, mn, rg)
    assert res["n_unique"] == want["n_unique"], c
    if want["n_unique"] < 2:
        return
    assert (res["n_oct"], res["status"]) == (want["n_oct"], 0), c
    for key in STAGES:
        assert res[key].tobytes() == np.asarray(want[key]).tobytes(), (c, key)


def test_batch_matches_oracle_per_cloud():
    clouds, mins, ranges = mixed_clouds()
    b, pts, mn, rg = build_batch(clouds, mins, ranges)
    b.build(pts, mn, rg)
    counts = b.cloud_counts()
    for c, p in enumerate(clouds):
        check_cloud(b, counts, c, p, mins[c], ranges[c])


def test_batch_graph_replay_deterministic():
    clouds, mins, ranges = mixed_clouds(seed=1)
    b, pts, mn, rg = build_batch(clouds, mins, ranges)
    b.capture(pts, mn, rg)
    b.replay()
    counts = b.cloud_counts()
    first = (b.counts.clone(), b.nodes.clone(), b.parent.clone())
    for _ in range(2):
        b.nodes.fill_(-1)  # slots past each cloud's M stay unwritten; M slots are rewritten
        b.replay()
        assert torch.equal(first[0], b.counts)
        for c in range(len(clouds)):
            ns, m = int(b.node_start[c]), int(counts[c][2])
            assert torch.equal(first[1][ns:ns + m], b.nodes[ns:ns + m]), c
        assert torch.equal(first[2], b.parent)
    for c in (0, 5, 12, 17, 30):
        check_cloud(b, counts, c, clouds[c], mins[c], ranges[c])


def test_batch_512_clouds_match_single_builds():
    """The batched workload's shape (512 clouds, sizes log-uniform, half
    uniform, half 8-Gaussian), scaled down 8x so every cloud is also checked
    against a single-cloud GPU build."""
    from pipeline_gb300 import datasets
    from pipeline_gb300.pipeline import OctreeBuilder

    clouds = datasets.batched(512, seed=11, lo=125, hi=125_000)
    mins = [0.0] * len(clouds)
    ranges = [1024.0] * len(clouds)
    b, pts, mn, rg = build_batch(clouds, mins, ranges)
    b.build(pts, mn, rg)
    counts = b.cloud_counts()
    single = OctreeBuilder(max(len(c) for c in clouds))
    for c in range(0, 512, 7):
        single.build(torch.from_numpy(clouds[c]).cuda(), 0.0, 1024.0)
        want = single.result()
        got = b.cloud_result(c, counts)
        assert (got["n_unique"], got["n_oct"]) == (want["n_unique"], want["n_oct"]), c
        for key in STAGES:
            assert got[key].tobytes() == np.asarray(want[key]).tobytes(), (c, key)


def test_work_queue_and_static_tiles_give_the_same_batch():
    """The batched octree-stage kernels run from an atomic work queue
    (persistent CTAs) or one CTA per tile; both equal the oracle."""
    from pipeline_gb300 import _lib

    lib = _lib.load()
    clouds, mins, ranges = mixed_clouds(seed=4)
    results = []
    try:
        for on in (0, 1):
            assert lib.oct_set_batch_work_queue(on) == _lib.OCT_OK
            b, pts, mn, rg = build_batch(clouds, mins, ranges)
            b.build(pts, mn, rg)
            results.append(b)
    finally:
        lib.oct_set_batch_work_queue(0)
    assert results[0].same_results(results[1])
    counts = results[1].cloud_counts()
    for c in range(0, len(clouds), 3):
        check_cloud(results[1], counts, c, clouds[c], mins[c], ranges[c])
    assert lib.oct_set_batch_work_queue(2) == _lib.OCT_ERR_INVALID_ARG
