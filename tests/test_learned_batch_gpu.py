"""Learned + batched build: one learned CDF shared by a batch of clouds drives
stage 2 (per-cloud learned buckets, sorted in shared memory), and every cloud
must still equal the oracle's build of it (apps/cpu_demo/main.cpp:72-154) and
the plain batched build, byte for byte, on the learned path and on its LSD
fall-back alike."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

STAGES = ["sorted_unique", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent",
          "edge_count", "prefix_sum", "oct_nodes"]


def _fit(clouds, mins, ranges, nb, segments=1024):
    from pipeline_gb300.kernels import k_ComputeMortonCode
    from pipeline_gb300.learned import LearnedCDF

    codes = []
    for f, mn, rg in zip(clouds, mins, ranges):
        if len(f) == 0:
            continue
        k = torch.empty(len(f), dtype=torch.int32, device="cuda")
        k_ComputeMortonCode(torch.from_numpy(np.ascontiguousarray(f)).cuda(), k, len(f), mn, rg)
        codes.append(k)
    return LearnedCDF(max_segments=segments).fit(torch.cat(codes), n_segments=segments, steps=100,
                                                 lr=0.05, n_buckets=nb)


def _build(clouds, mins, ranges, model=None, nb=None):
    from pipeline_gb300.batch import BatchOctreeBuilder

    sizes = [len(c) for c in clouds]
    b = BatchOctreeBuilder(sizes, model=model, n_buckets=nb)
    pts = torch.from_numpy(np.concatenate(clouds, 0)).cuda()
    mn = torch.tensor(mins, dtype=torch.float32, device="cuda")
    rg = torch.tensor(ranges, dtype=torch.float32, device="cuda")
    return b, pts, mn, rg


def _check_all(b, clouds, mins, ranges):
    counts = b.cloud_counts()
    for c, p in enumerate(clouds):
        got = b.cloud_result(c, counts)
        want = O.build_all(p, mins[c], ranges[c])
        assert got["n_unique"] == want["n_unique"], c
        if want["n_unique"] < 2:
            continue
        assert (got["n_oct"], got["status"]) == (want["n_oct"], 0), c
        for key in STAGES:
            assert np.asarray(got[key]).tobytes() == np.asarray(want[key]).tobytes(), (c, key)


@pytest.fixture(scope="module")
def frames():
    from pipeline_gb300 import datasets

    return datasets.scan_frames(40, seed=5)


def test_frames_learned_batched_matches_oracle_and_plain(frames):
    fr, mins, ranges = frames
    model = _fit(fr[:8], mins[:8], ranges[:8], nb=64)
    test = fr[8:]
    b, pts, mn, rg = _build(test, mins[8:], ranges[8:], model, 64)
    b.build(pts, mn, rg)
    st = b.learned_stats()
    assert st["fallback"] == 0 and st["max_bucket"] > 0, st
    _check_all(b, test, mins[8:], ranges[8:])
    plain, pts2, mn2, rg2 = _build(test, mins[8:], ranges[8:])
    plain.build(pts2, mn2, rg2)
    torch.cuda.synchronize()
    assert plain.same_results(b)


def test_learned_batched_falls_back_when_a_bucket_fits_no_form(frames):
    """One bucket per frame: far more unique keys than the bitonic form holds,
    over a span wider than the bitmap form covers, so the LSD passes run."""
    fr, mins, ranges = frames
    model = _fit(fr[:4], mins[:4], ranges[:4], nb=1, segments=64)
    test = fr[30:36]
    b, pts, mn, rg = _build(test, mins[30:36], ranges[30:36], model, 1)
    b.build(pts, mn, rg)
    st = b.learned_stats()
    assert st["fallback"] == 1 and st["max_bucket"] > 16384, st
    _check_all(b, test, mins[30:36], ranges[30:36])


def test_mixed_clouds_learned_batched_and_graph_replay():
    from test_batch_gpu import mixed_clouds

    clouds, mins, ranges = mixed_clouds(seed=3)
    model = _fit(clouds, mins, ranges, nb=16, segments=256)
    b, pts, mn, rg = _build(clouds, mins, ranges, model, 16)
    b.capture(pts, mn, rg)
    b.replay()
    torch.cuda.synchronize()
    first = (b.counts.clone(), b.codes.clone())
    _check_all(b, clouds, mins, ranges)
    b.replay()
    torch.cuda.synchronize()
    assert torch.equal(first[0], b.counts) and torch.equal(first[1], b.codes)
