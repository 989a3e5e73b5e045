"""Learned bucketed sort + unique, and the whole learned build: bit-exact with
the plain path / the oracle; fallback exact; the trained model's gain over
plain key-space bucketing on clustered keys."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def dev_keys(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()


def fitted(keys_np, n_buckets=4096, segments=4096, steps=100, sample=1 << 18, seed=0):
    from pipeline_gb300.learned import LearnedCDF

    rng = np.random.default_rng(seed)
    samp = keys_np[rng.integers(0, len(keys_np), min(sample, len(keys_np)))]
    m = LearnedCDF(max_segments=segments)
    m.fit(dev_keys(samp), n_segments=segments, steps=steps, n_buckets=n_buckets)
    return m


def no_model(n_buckets=4096):
    """Key-space bucketing: one segment [0, 2^30) with a linear CDF (top key bits)."""
    from pipeline_gb300.learned import LearnedCDF

    m = LearnedCDF(max_segments=4)
    m.fit(dev_keys(np.array([0, (1 << 30) - 1], np.uint32)), n_segments=1, steps=0,
          n_buckets=n_buckets)
    return m


def clustered_keys(n, seed=3):
    from pipeline_gb300 import datasets

    pts = datasets.gaussian_mixture(n, 64, np.random.default_rng(seed), noise=0.05)
    return O.morton(pts, 0.0, 1024.0, threads=4)


@pytest.mark.parametrize("kind", ["uniform", "clustered"])
@pytest.mark.parametrize("n", [1, 5000, 1 << 20])
def test_lsort_unique_exact(kind, n):
    from pipeline_gb300.pipeline import lsort_unique

    if kind == "uniform":
        keys = np.random.default_rng(n).integers(0, 1 << 30, n).astype(np.uint32)
    else:
        keys = clustered_keys(n)
    m = fitted(keys, n_buckets=1024 if n < 100000 else 4096)
    out, stats = lsort_unique(dev_keys(keys), m)
    assert out.cpu().numpy().view(np.uint32).tobytes() == np.unique(keys).tobytes()
    assert stats["fallback"] == 0, stats


@pytest.mark.parametrize("n", [1023, 1025, 155_649, 466_945, 1_089_537, 1_245_185, 2_000_001])
def test_lsort_unique_tile_shapes(n):
    """The one-pass bin sizes its tiles to the input (up to 16,384 keys, any
    length, the same number per SM): sizes below and around those steps, with
    partial last tiles and runs of equal keys (which the bin leaves out of
    the buckets)."""
    from pipeline_gb300.pipeline import lsort_unique

    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << 30, n).astype(np.uint32)
    keys[5::9] = keys[4::9][: len(keys[5::9])]  # equal neighbours
    m = fitted(keys, n_buckets=1024)
    out, stats = lsort_unique(dev_keys(keys), m)
    assert out.cpu().numpy().view(np.uint32).tobytes() == np.unique(keys).tobytes()
    assert stats["fallback"] == 0, stats


def test_lsort_forced_fallback_is_exact():
    from pipeline_gb300.pipeline import lsort_unique

    keys = clustered_keys(1 << 20)
    m = fitted(keys)
    out, stats = lsort_unique(dev_keys(keys), m, overflow_threshold=-1.0)
    assert stats["fallback"] == 1 and stats["skip"] == 1
    assert out.cpu().numpy().view(np.uint32).tobytes() == np.unique(keys).tobytes()


def test_bucket_past_bin_capacity_falls_back_exact():
    """A model applied to keys it was not fit on: bucket 0 receives far more
    keys than a bucket range of the one-pass bin holds (16,384 here), so the
    sort falls back to the LSD passes, and the result is still exact."""
    from pipeline_gb300.pipeline import lsort_unique

    rng = np.random.default_rng(17)
    m = fitted(rng.integers(0, 1 << 30, 1 << 20).astype(np.uint32), n_buckets=1024)
    keys = rng.integers(0, 1 << 19, 300_000).astype(np.uint32)  # all in bucket 0
    out, stats = lsort_unique(dev_keys(keys), m)
    assert stats["fallback"] == 1 and stats["skip"] == 1, stats
    assert stats["max_bucket"] > 16384, stats
    assert out.cpu().numpy().view(np.uint32).tobytes() == np.unique(keys).tobytes()


def test_trained_model_balances_buckets_where_key_bits_do_not():
    """What the trained CDF gains over bucketing by key bits on clustered keys:
    the largest bucket and the share of keys in oversized buckets."""
    from pipeline_gb300.pipeline import lsort_unique

    keys = clustered_keys(1 << 22)
    trained = fitted(keys)
    plain = no_model()
    out_t, st_t = lsort_unique(dev_keys(keys), trained, overflow_threshold=1.0)
    out_p, st_p = lsort_unique(dev_keys(keys), plain, overflow_threshold=1.0)
    want = np.unique(keys).tobytes()
    assert out_t.cpu().numpy().view(np.uint32).tobytes() == want
    assert out_p.cpu().numpy().view(np.uint32).tobytes() == want
    avg = len(keys) / 4096
    assert st_t["fallback"] == 0, st_t
    assert st_t["max_bucket"] < 8 * avg, st_t
    assert st_p["max_bucket"] > 10 * st_t["max_bucket"], (st_p, st_t)
    assert st_t["overflow_frac"] < 0.05 < st_p["overflow_frac"], (st_t, st_p)


@pytest.mark.parametrize("kind", ["uniform", "clustered"])
def test_learned_build_matches_oracle(kind):
    from pipeline_gb300 import datasets
    from pipeline_gb300.pipeline import LearnedOctreeBuilder

    n = 1 << 20
    if kind == "uniform":
        pts = O.init_random_vec4(n)
    else:
        pts = datasets.gaussian_mixture(n, 64, np.random.default_rng(9), noise=0.05)
    keys = O.morton(pts, 0.0, 1024.0)
    m = fitted(keys)
    b = LearnedOctreeBuilder(n, m)
    b.build(torch.from_numpy(pts).cuda(), 0.0, 1024.0)
    res = b.result()
    want = O.build_all(pts, 0.0, 1024.0, threads=4)
    assert (res["n_unique"], res["n_oct"], res["status"]) == (want["n_unique"], want["n_oct"], 0)
    for key in ["sorted_unique", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child",
                "parent", "edge_count", "prefix_sum", "oct_nodes"]:
        assert res[key].tobytes() == np.asarray(want[key]).tobytes(), key
    assert b.lsort_stats()["fallback"] == 0


def test_learned_build_with_a_foreign_model_falls_back_exact():
    """A learned build from points whose codes all fall in one bucket of the
    model (fit on uniform codes): the one-pass bin overflows that bucket's
    range, the build takes the fallback sort and still equals the oracle."""
    from pipeline_gb300.pipeline import LearnedOctreeBuilder

    rng = np.random.default_rng(23)
    m = fitted(rng.integers(0, 1 << 30, 1 << 20).astype(np.uint32), n_buckets=1024)
    n = 300_000
    pts = np.zeros((n, 4), np.float32)
    pts[:, :3] = rng.uniform(0.0, 60.0, (n, 3))  # codes below 2^18: bucket 0
    pts[:, 3] = 1.0
    b = LearnedOctreeBuilder(n, m)
    b.build(torch.from_numpy(pts).cuda(), 0.0, 1024.0)
    res = b.result()
    st = b.lsort_stats()
    assert st["fallback"] == 1 and st["max_bucket"] > 16384, st
    want = O.build_all(pts, 0.0, 1024.0, threads=4)
    assert (res["n_unique"], res["n_oct"], res["status"]) == (want["n_unique"], want["n_oct"], 0)
    for key in ["sorted_unique", "left_child", "parent", "prefix_sum", "oct_nodes"]:
        assert res[key].tobytes() == np.asarray(want[key]).tobytes(), key


@pytest.mark.parametrize("form", ["bitmap", "radix", "bitonic", "wide_bitmap"])
def test_each_bucket_form_exact(form):
    """Inputs chosen so the buckets take one shared-memory form: dense keys
    (bitmap), sparse keys in small buckets (radix sort), sparse keys in
    buckets of 8K-16K keys (bitonic), dense buckets of more than 8K keys
    (whole-region bitmap). Duplicates included; result = np.unique."""
    from pipeline_gb300.pipeline import lsort_unique

    rng = np.random.default_rng(len(form))
    if form == "bitmap":  # 256 keys per bucket over spans of ~1K keys
        keys = rng.integers(0, 1 << 22, 1 << 20).astype(np.uint32)
        m, want = fitted(keys, n_buckets=4096), "bitmap_buckets"
    elif form == "radix":  # 256 keys per bucket over spans of 2^18
        keys = rng.integers(0, 1 << 30, 1 << 20).astype(np.uint32)
        m, want = no_model(4096), "radix_buckets"
    elif form == "bitonic":  # ~12K keys per bucket over spans of 2^22
        keys = rng.integers(0, 1 << 30, 12_000 * 256).astype(np.uint32)
        m, want = no_model(256), "bitonic_buckets"
    else:  # ~12K keys per bucket over spans of ~8K
        keys = rng.integers(0, 1 << 21, 12_000 * 256).astype(np.uint32)
        m, want = fitted(keys, n_buckets=256), "bitmap_buckets"
    n7 = len(keys[1::7])
    keys[1::7] = keys[:n7]  # duplicates across the array
    out, st = lsort_unique(dev_keys(keys), m, overflow_threshold=1.0)
    assert out.cpu().numpy().view(np.uint32).tobytes() == np.unique(keys).tobytes()
    assert st["fallback"] == 0 and st["failed_buckets"] == 0, st
    assert st[want] >= 0.9 * m.n_buckets, st


@pytest.mark.parametrize("cfg", [(10, 16, 16, 0), (10, 16, 16, 1), (10, 16, 24, 1), (8, 16, 16, 0),
                                 (8, 16, 24, 1)])
def test_every_sort_config_sorts(cfg):
    from pipeline_gb300 import _lib
    from pipeline_gb300.kernels import k_SimpleRadixSort

    import ctypes

    lib = _lib.load()
    old = (ctypes.c_int * 4)()
    lib.oct_get_sort_config(old)
    try:
        assert lib.oct_set_sort_config(*cfg) == 0
        rng = np.random.default_rng(sum(cfg))
        for n, bits in [(1_000_003, 30), (300_001, 32), (7, 30)]:
            a = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
            keys = dev_keys(a)
            k_SimpleRadixSort(keys, n, key_bits=bits)
            assert keys.cpu().numpy().view(np.uint32).tobytes() == np.sort(a).tobytes(), (cfg, n, bits)
    finally:
        lib.oct_set_sort_config(*list(old))
