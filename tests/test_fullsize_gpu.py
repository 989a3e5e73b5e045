"""The spec workloads at full size, every stage buffer against the oracle.

  clustered   16,777,216 points, 64 anisotropic Gaussians + 5% noise (seed 7):
              the plain whole build (which takes the LSD form of stages 2-3 on
              this uneven cloud) and the learned build (model fit on 262,144
              sampled Morton codes of the cloud, as the bench does);
  batched     all 512 clouds of the batched workload (sizes log-uniform in
              [1K, 1M], seed 11; 69.3M points) in one batched build;
  frames      scan-like frames (seed 5), frames 32-255 with their own min and
              range: in one batched build, and one by one through the learned
              build with a model fit only on frames 0-31's Morton codes.

The oracle (oracle/oracle.c) runs stages 1-6 on all host cores and stages 7-8
on one thread (the reference's sequential semantics); the reference behaviour
is apps/cpu_demo/main.cpp:72-154.
"""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

STAGES = ["sorted_unique", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent",
          "edge_count", "prefix_sum", "oct_nodes"]
THREADS = max(1, min(16, os.cpu_count() or 1))


def _same(got, want, where):
    assert (got["n_unique"], got["n_oct"]) == (want["n_unique"], want["n_oct"]), where
    assert got.get("status", 0) == 0, where
    for key in STAGES:
        g, w = np.asarray(got[key]), np.asarray(want[key])
        assert g.tobytes() == w.tobytes(), (where, key)


@pytest.fixture(scope="module")
def frames():
    from pipeline_gb300 import datasets

    return datasets.scan_frames(256, seed=5)


def _fit(sample_keys, segments, nb):
    from pipeline_gb300.learned import LearnedCDF

    return LearnedCDF(max_segments=segments).fit(sample_keys, n_segments=segments, steps=100,
                                                 lr=0.05, n_buckets=nb)


def test_clustered_16m_plain_and_learned_match_oracle():
    from pipeline_gb300 import datasets
    from pipeline_gb300.kernels import k_ComputeMortonCode
    from pipeline_gb300.pipeline import LearnedOctreeBuilder, OctreeBuilder

    n = 1 << 24
    pts_h = datasets.clustered(n, seed=7)
    want = O.build_all(pts_h, 0.0, 1024.0, threads=THREADS)
    pts = torch.from_numpy(pts_h).cuda()
    plain = OctreeBuilder(n)
    plain.build(pts, 0.0, 1024.0)
    _same(plain.result(), want, "plain")
    del plain
    idx = torch.from_numpy(np.random.default_rng(1).integers(0, n, 1 << 18)).cuda()
    sample_keys = torch.empty(1 << 18, dtype=torch.int32, device="cuda")
    k_ComputeMortonCode(pts.index_select(0, idx).contiguous(), sample_keys, 1 << 18, 0.0, 1024.0)
    learned = LearnedOctreeBuilder(n, _fit(sample_keys, 4096, 4096))
    learned.build(pts, 0.0, 1024.0)
    st = learned.lsort_stats()
    _same(learned.result(), want, "learned")
    assert st["fallback"] == 0, st  # the model's buckets, not the fallback, made the result


def test_batched_512_every_cloud_matches_oracle():
    from pipeline_gb300 import datasets
    from pipeline_gb300.batch import BatchOctreeBuilder

    clouds = datasets.batched(512, seed=11)
    sizes = [len(c) for c in clouds]
    b = BatchOctreeBuilder(sizes)
    pts = torch.from_numpy(np.concatenate(clouds, 0)).cuda()
    mins = torch.zeros(len(clouds), dtype=torch.float32, device="cuda")
    ranges = torch.full((len(clouds),), 1024.0, dtype=torch.float32, device="cuda")
    b.capture(pts, mins, ranges)
    b.replay()
    counts = b.cloud_counts()
    for c, p in enumerate(clouds):
        _same(b.cloud_result(c, counts), O.build_all(p, 0.0, 1024.0, threads=THREADS), f"cloud {c}")


def test_frames_32_255_batched_and_learned_match_oracle(frames):
    from pipeline_gb300.batch import BatchOctreeBuilder
    from pipeline_gb300.kernels import k_ComputeMortonCode
    from pipeline_gb300.pipeline import LearnedOctreeBuilder

    fr, mins, ranges = frames
    codes = []
    for f, mn, rg in zip(fr[:32], mins[:32], ranges[:32]):
        k = torch.empty(len(f), dtype=torch.int32, device="cuda")
        k_ComputeMortonCode(torch.from_numpy(f).cuda(), k, len(f), mn, rg)
        codes.append(k)
    nb = 512
    model = _fit(torch.cat(codes), 1024, nb)
    test_f = fr[32:]
    sizes = [len(f) for f in test_f]
    b = BatchOctreeBuilder(sizes)
    pts = torch.from_numpy(np.concatenate(test_f, 0)).cuda()
    b.build(pts, torch.tensor(mins[32:], dtype=torch.float32, device="cuda"),
            torch.tensor(ranges[32:], dtype=torch.float32, device="cuda"))
    counts = b.cloud_counts()
    learned = LearnedOctreeBuilder(max(sizes), model, n_buckets=nb)
    for i, (f, mn, rg) in enumerate(zip(test_f, mins[32:], ranges[32:])):
        want = O.build_all(f, mn, rg, threads=THREADS)
        _same(b.cloud_result(i, counts), want, f"batched frame {32 + i}")
        learned.build(torch.from_numpy(f).cuda(), mn, rg)
        _same(learned.result(), want, f"learned frame {32 + i}")
