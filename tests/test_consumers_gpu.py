"""Device input generator, Morton decode and the octree check against the
oracle (oracle/oracle.c restates the reference's device generator, its
morton32_to_xyz and its checkTree)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,mn,rg,seed", [(1, 0.0, 1024.0, 114514), (767, 0.0, 1024.0, 114514),
                                          (100_003, 0.0, 1024.0, 114514), (5000, -3.5, 7.25, 1),
                                          (4099, 100.0, 0.001, -17), (3000, 0.0, 1.0, 0)])
def test_device_generator_matches_oracle(n, mn, rg, seed):
    from pipeline_gb300.kernels import k_InitRandomVec4_device

    pts = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    k_InitRandomVec4_device(pts, n, mn, rg, seed)
    want = O.init_random_vec4_gpu(n, mn, rg, seed)
    assert pts.cpu().numpy().tobytes() == want.tobytes()


def test_device_generated_cloud_builds_like_the_oracle():
    from pipeline_gb300.kernels import k_InitRandomVec4_device
    from pipeline_gb300.pipeline import OctreeBuilder

    n = 200_000
    pts = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    k_InitRandomVec4_device(pts, n, 0.0, 1024.0, 114514)
    b = OctreeBuilder(n)
    b.build(pts, 0.0, 1024.0)
    res = b.result()
    want = O.build_all(pts.cpu().numpy(), 0.0, 1024.0, threads=4)
    assert (res["n_unique"], res["n_oct"]) == (want["n_unique"], want["n_oct"])
    assert res["oct_nodes"].tobytes() == want["oct_nodes"].tobytes()


def test_morton_decode_matches_oracle():
    from pipeline_gb300.kernels import morton_decode

    rng = np.random.default_rng(2)
    codes = np.concatenate([rng.integers(0, 1 << 30, 50_000), [0, (1 << 30) - 1, 7]]).astype(np.uint32)
    for mn, rg in [(0.0, 1024.0), (-37.3, 129.0000153), (5.0, 0.125)]:
        got = morton_decode(torch.from_numpy(codes.view(np.int32)).cuda(), len(codes), mn, rg)
        assert got.cpu().numpy().tobytes() == O.morton_decode(codes, mn, rg).tobytes()


def _root(res):
    codes = res["sorted_unique"]
    level = int(res["prefix_n"][0]) // 3
    return int(codes[0]) >> (30 - 3 * level), 3 * level


@pytest.mark.parametrize("kind", ["uniform", "clustered"])
def test_check_tree_on_built_octrees(kind):
    from pipeline_gb300 import datasets
    from pipeline_gb300.kernels import check_tree
    from pipeline_gb300.pipeline import OctreeBuilder

    n = 300_000
    if kind == "uniform":
        pts = O.init_random_vec4(n)
    else:
        pts = datasets.gaussian_mixture(n, 16, np.random.default_rng(1), noise=0.05)
    b = OctreeBuilder(n)
    b.build(torch.from_numpy(pts).cuda(), 0.0, 1024.0)
    res = b.result()
    prefix, clen = _root(res)
    got = check_tree(b.nodes, res["n_oct"], b.codes, res["n_unique"], prefix, clen)
    want = O.check_tree(res["oct_nodes"], res["sorted_unique"], prefix, clen)
    assert got == want
    assert got[0] >= 1 and got[2] == 0


def test_check_tree_finds_wrong_leaves_and_bad_links():
    """Leaf-mask bits pointing at keys of another cell, child indices out of
    range: the GPU counts equal the oracle's on the same (altered) octree."""
    from pipeline_gb300.kernels import check_tree
    from pipeline_gb300.pipeline import OctreeBuilder

    n = 50_000
    pts = O.init_random_vec4(n, seed=3)
    b = OctreeBuilder(n)
    b.build(torch.from_numpy(pts).cuda(), 0.0, 1024.0)
    res = b.result()
    nodes = res["oct_nodes"].copy()
    m, u = len(nodes), res["n_unique"]
    rng = np.random.default_rng(9)
    for p in rng.integers(0, m, 400):
        c = int(rng.integers(0, 8))
        nodes[p]["child_leaf_mask"] |= 1 << c
        nodes[p]["children"][c] = int(rng.integers(0, u))
    for p in rng.integers(0, m, 50):
        c = int(rng.integers(0, 8))
        nodes[p]["child_node_mask"] |= 1 << c
        nodes[p]["children"][c] = m + 5
    prefix, clen = _root(res)
    want = O.check_tree(nodes, res["sorted_unique"], prefix, clen)
    dev_nodes = torch.from_numpy(nodes.view(np.int32).reshape(-1, 15).copy()).cuda()
    got = check_tree(dev_nodes, m, b.codes, u, prefix, clen)
    assert got == want
    assert want[1] > 0 and want[2] > 0 and want[3] > 0


@pytest.mark.parametrize("n", [1, 767, 100_003, 1 << 22])
def test_init_sequences(n):
    from pipeline_gb300.kernels import k_InitAscending, k_InitDescending

    d = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    a = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    k_InitDescending(d, n)
    k_InitAscending(a, n)
    idx = np.arange(n, dtype=np.int64)
    assert np.array_equal(d.cpu().numpy().view(np.uint32).astype(np.int64), n - idx)
    assert np.array_equal(a.cpu().numpy().view(np.uint32).astype(np.int64), idx)


def _device_init_fixture():
    import json
    import os

    path = os.path.join(os.path.dirname(__file__), "golden", "device_init.json")
    if not os.path.exists(path):
        return []
    with open(path) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", _device_init_fixture(), ids=lambda c: f'n{c["n"]}_seed{c["seed"]}')
def test_device_generator_matches_reference_gpu_output(case):
    """oct_init_random_vec4_device against the reference's own kernel's output
    (kernels/cuda/00_init.cu run on a GB300: tests/golden/device_init.json)."""
    from pipeline_gb300.kernels import k_InitRandomVec4_device

    n = case["n"]
    pts = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    k_InitRandomVec4_device(pts, n, case["min"], case["range"], case["seed"])
    assert O.fnv1a64(pts.cpu().numpy()) == case["hash"]
