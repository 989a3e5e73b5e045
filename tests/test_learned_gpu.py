"""Learned CDF model: GPU forward/backward against the fp64 CPU reference
(oracle/learned_ref.py), exact bucket ids, training lowers the loss, and the
model survives a save/load round trip."""
import numpy as np
import pytest
import torch

from oracle import learned_ref as LR

pytestmark = pytest.mark.gpu


def clustered_keys(n, seed=3):
    from oracle import oracle as O
    from pipeline_gb300 import datasets

    pts = datasets.gaussian_mixture(n, 16, np.random.default_rng(seed), noise=0.05)
    return O.morton(pts, 0.0, 1024.0)


def model_on(sample_sorted, segments=256, steps=0, nb=1024):
    from pipeline_gb300.learned import LearnedCDF

    m = LearnedCDF(max_segments=segments)
    m.fit(torch.from_numpy(sample_sorted.view(np.int32)).cuda(), n_segments=segments, steps=steps,
          n_buckets=nb)
    return m


def test_knots_match_reference():
    keys = np.sort(clustered_keys(50_000))
    m = model_on(keys, segments=256)
    t = m.tables()
    assert np.array_equal(t["x"], LR.knots_from_sorted_sample(keys, 256))


@pytest.mark.parametrize("seed", [0, 1])
def test_loss_and_gradient_match_fp64_reference(seed):
    keys = np.sort(clustered_keys(40_000, seed=seed + 10))
    m = model_on(keys, segments=128)
    x = m.tables()["x"]
    theta = np.random.default_rng(seed).normal(0.5, 0.4, len(x) - 1).astype(np.float32)
    m.set_theta(theta)
    loss, grad = m.loss_grad(torch.from_numpy(keys.view(np.int32)).cuda())
    L_ref, g_ref = LR.loss_and_grad(theta.astype(np.float64), keys, x)
    # float32 forward/backward vs fp64: relative tolerance on the loss, and on
    # the gradient relative to its largest component.
    assert abs(loss - L_ref) <= 2e-3 * L_ref + 1e-9
    scale = np.max(np.abs(g_ref))
    assert np.max(np.abs(grad - g_ref)) <= 2e-3 * scale


def test_reference_gradient_matches_finite_differences():
    keys = np.sort(clustered_keys(5000).astype(np.int64))
    x = LR.knots_from_sorted_sample(keys, 32)
    theta = np.random.default_rng(7).normal(0.5, 0.3, len(x) - 1)
    _, g = LR.loss_and_grad(theta, keys, x)
    eps = 1e-6
    for mi in range(0, len(theta), 5):
        tp, tm = theta.copy(), theta.copy()
        tp[mi] += eps
        tm[mi] -= eps
        fd = (LR.loss_and_grad(tp, keys, x)[0] - LR.loss_and_grad(tm, keys, x)[0]) / (2 * eps)
        assert abs(fd - g[mi]) <= 1e-6 * np.max(np.abs(g)) + 1e-12


def test_training_lowers_loss():
    keys = np.sort(clustered_keys(60_000))
    m0 = model_on(keys, segments=256, steps=0)
    m1 = model_on(keys, segments=256, steps=150)
    assert m1.header()["steps"] == 150
    assert m1.header()["loss"] < m0.header()["loss"]


def test_training_recovers_from_a_perturbed_model():
    """From heights far from the data's CDF, the GPU forward/backward + Adam
    steps bring the loss down by orders of magnitude (the fp64 reference's own
    Adam loop on the same start goes the same way)."""
    import ctypes as C

    from pipeline_gb300 import _lib

    keys = np.sort(clustered_keys(60_000))
    m = model_on(keys, segments=128, steps=0)
    x = m.tables()["x"]
    theta0 = np.random.default_rng(4).normal(0.0, 2.0, len(x) - 1).astype(np.float32)
    m.set_theta(theta0)
    lib = _lib.load()
    sample = torch.from_numpy(keys.view(np.int32)).cuda()
    loss0, _ = m.loss_grad(sample)
    # 200 GPU Adam steps on the perturbed parameters through the training kernels
    for _ in range(200):
        rc = lib.oct_lcdf_train_steps(C.c_void_p(sample.data_ptr()), sample.numel(),
                                      C.c_void_p(m.blob.data_ptr()), m.max_segments, 1, 0.05,
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0
    loss1, _ = m.loss_grad(sample)
    _, hist = LR.adam_fit(keys, x, steps=200, lr=0.05, theta0=theta0.astype(np.float64))
    assert loss1 < 0.1 * loss0
    assert loss1 < 3 * hist[-1] + 1e-9


def test_buckets_exact_and_monotone():
    keys = np.sort(clustered_keys(80_000))
    m = model_on(keys, segments=256, steps=50, nb=1024)
    t = m.tables()
    probe = np.random.default_rng(1).integers(0, 1 << 30, 200_000).astype(np.uint32)
    probe = np.concatenate([probe, keys.astype(np.uint32), np.array([0, (1 << 30) - 1], np.uint32)])
    got = m.buckets(torch.from_numpy(probe.view(np.int32)).cuda()).cpu().numpy()
    want = LR.buckets(probe, t["x"], t["yq"], t["slope"], 1024)
    assert np.array_equal(got, want)
    order = np.argsort(probe, kind="stable")
    assert np.all(np.diff(got[order]) >= 0)
    assert got.min() >= 0 and got.max() <= 1023


def test_bucket_boundaries_match_reference():
    """The boundary table the bucketed sort searches: bounds[b] is the smallest
    key whose bucket is >= b, blut[p] the bucket of key p << 16 (CPU reference
    buckets on the same fixed-point tables)."""
    keys = np.sort(clustered_keys(80_000))
    nb = 1024
    m = model_on(keys, segments=256, steps=30, nb=nb)
    t = m.tables()
    bounds, blut = t["bounds"], t["blut"]
    assert bounds[0] == 0 and bounds[nb] == 1 << 30
    assert np.all(np.diff(bounds) >= 0)
    inner = bounds[1:nb]
    reach = inner < (1 << 30)
    at = LR.buckets(inner[reach].astype(np.uint32), t["x"], t["yq"], t["slope"], nb)
    assert np.all(at >= np.arange(1, nb)[reach])
    before = LR.buckets((inner[reach] - 1).astype(np.uint32), t["x"], t["yq"], t["slope"], nb)
    assert np.all(before < np.arange(1, nb)[reach])
    top = LR.buckets(np.array([(1 << 30) - 1], np.uint32), t["x"], t["yq"], t["slope"], nb)[0]
    assert np.all(np.arange(1, nb)[~reach] > top)
    cells = np.minimum(np.arange((1 << 14) + 1, dtype=np.int64) << 16, (1 << 30) - 1)
    want = LR.buckets(cells.astype(np.uint32), t["x"], t["yq"], t["slope"], nb)
    assert np.array_equal(blut, want)


def test_state_dict_round_trip():
    from pipeline_gb300.learned import LearnedCDF

    keys = np.sort(clustered_keys(20_000))
    m = model_on(keys, segments=64, steps=20, nb=256)
    sd = m.state_dict()
    m2 = LearnedCDF.from_state_dict(sd)
    probe = torch.from_numpy(keys.view(np.int32)).cuda()
    assert torch.equal(m.buckets(probe), m2.buckets(probe))
    assert m2.header()["steps"] == 20
