"""GPU parity: every stage through the C ABI, byte for byte against the oracle
and the reference-generated fixtures in tests/golden/.

Integer and byte outputs must be identical; the float fields (OctNode corner
and cell_size) are compared bit for bit as well, since the kernels reproduce
the reference's FP32 operation order with no contraction.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

STAGES = ["sorted_unique", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent",
          "edge_count", "prefix_sum", "oct_nodes"]
GARBAGE = 0x5A


def K():
    from pipeline_gb300 import kernels

    return kernels


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.view(dtype)
    return t.cuda()


def u32(t):
    return t.cpu().numpy().view(np.uint32)


def garbage(n, dtype):
    return torch.full((max(n, 1),), GARBAGE, dtype=torch.uint8, device="cuda").view(dtype) if dtype == torch.uint8 \
        else torch.full((max(n, 1),), 0x5A5A5A5A, dtype=torch.int32, device="cuda")


# --------------------------------------------------------------- stage 1 --
def test_morton_small_cases(small_cases):
    k = K()
    for name, case in small_cases.items():
        pts = dev(case["points"])
        n = len(case["points"])
        out = torch.empty(n, dtype=torch.int32, device="cuda")
        k.k_ComputeMortonCode(pts, out, n, 0.0, 1024.0)
        assert u32(out).tobytes() == case["morton"].tobytes(), name


def test_morton_cfg1_hash(golden):
    k = K()
    g = golden["cfg1_uniform_1m"]
    pts = k.k_InitRandomVec4(None, g["n"], g["min"], g["range"], g["seed"])
    out = torch.empty(g["n"], dtype=torch.int32, device="cuda")
    k.k_ComputeMortonCode(dev(pts), out, g["n"], g["min"], g["range"])
    assert O.fnv1a64(u32(out)) == g["hashes"]["morton"]


def test_morton_nonzero_min_matches_oracle():
    """Frames quantise with min != 0: the FP32 order (sub, div, mul) matters."""
    k = K()
    rng = np.random.default_rng(5)
    pts = rng.uniform(-37.3, 91.7, (100_003, 4)).astype(np.float32)
    mn, rg = np.float32(-37.3), np.float32(129.0000153)
    out = torch.empty(len(pts), dtype=torch.int32, device="cuda")
    k.k_ComputeMortonCode(dev(pts), out, len(pts), float(mn), float(rg))
    assert u32(out).tobytes() == O.morton(pts, float(mn), float(rg)).tobytes()


@pytest.mark.parametrize("mn,rg", [(0.0, 1024.0), (-37.3, 129.0000153), (1e-3, 3.0e-2),
                                   (-5000.0, 9999.5), (0.25, 1.0)])
def test_morton_cell_boundaries_match_oracle(mn, rg):
    """Coordinates on and a few ulps either side of every cell boundary
    min + k * range / 1024 (where the quotient's last bit decides the cell),
    plus random ones: codes equal the oracle's IEEE-division encode."""
    k = K()
    mn, rg = np.float32(mn), np.float32(rg)
    cells = np.arange(1025, dtype=np.float64)
    base = (mn.astype(np.float64) + cells * rg.astype(np.float64) / 1024.0).astype(np.float32)
    vals = [base]
    for steps in (1, 2, 3):
        up, down = base.copy(), base.copy()
        for _ in range(steps):
            up = np.nextafter(up, np.float32(np.inf))
            down = np.nextafter(down, np.float32(-np.inf))
        vals += [up, down]
    v = np.concatenate(vals)
    v = v[(v >= mn) & (v <= np.float32(mn + rg))]
    rng = np.random.default_rng(int(abs(mn) * 1000) + 7)
    n = 3 * len(v) + 200_000
    pts = rng.uniform(float(mn), float(mn + rg), (n, 4)).astype(np.float32)
    for axis in range(3):  # every boundary value on every axis
        pts[axis * len(v):(axis + 1) * len(v), axis] = v
    pts = np.clip(pts, mn, np.float32(mn + rg))
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    k.k_ComputeMortonCode(dev(pts), out, n, float(mn), float(rg))
    assert u32(out).tobytes() == O.morton(pts, float(mn), float(rg)).tobytes()


def test_morton_range_status():
    k = K()
    pts = np.zeros((1000, 4), np.float32)
    pts[17, 1] = -5.0
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.empty(1000, dtype=torch.int32, device="cuda")
    k.k_ComputeMortonCode(dev(pts), out, 1000, 0.0, 1024.0, status=st)
    assert int(st.item()) & 4
    st.zero_()
    pts[17, 1] = 1024.0  # x == min + range is in the reference's domain (wraps to 0)
    k.k_ComputeMortonCode(dev(pts), out, 1000, 0.0, 1024.0, status=st)
    assert int(st.item()) == 0


# --------------------------------------------------------------- stage 2 --
def test_sort_kat(golden):
    """tests/xmake.lua:9-13 through the GPU sort, both digit widths."""
    k = K()
    kat = golden["kat_sort"]
    for bits in (32, 30):
        keys = dev(np.array(kat["input"], np.uint32), torch.int32)
        k.k_SimpleRadixSort(keys, len(kat["input"]), key_bits=bits)
        assert u32(keys).tolist() == kat["expected"]


@pytest.mark.parametrize("n", [0, 1, 2, 3, 31, 1000, 7679, 7680, 7681, 8191, 8192, 8193,
                               65536 * 3 + 17, 1 << 20, (1 << 22) + 5])
@pytest.mark.parametrize("bits", [32, 30])
def test_sort_random(n, bits):
    k = K()
    rng = np.random.default_rng(n * 7 + bits)
    hi = 1 << bits
    a = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    keys = dev(a, torch.int32)
    alt = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    k.k_SimpleRadixSort(keys, alt, n, key_bits=bits, status=st)
    assert u32(keys).tobytes() == np.sort(a).tobytes()
    assert int(st.item()) == 0


@pytest.mark.parametrize("pattern", ["equal", "sorted", "reversed", "two_values", "few_bins"])
def test_sort_patterns(pattern):
    k = K()
    n = 300_001
    rng = np.random.default_rng(3)
    if pattern == "equal":
        a = np.full(n, 0x2ABCDEF, np.uint32)
    elif pattern == "sorted":
        a = np.sort(rng.integers(0, 1 << 30, n).astype(np.uint32))
    elif pattern == "reversed":
        a = np.sort(rng.integers(0, 1 << 30, n).astype(np.uint32))[::-1].copy()
    elif pattern == "two_values":
        a = np.where(rng.random(n) < 0.5, 5, (1 << 30) - 1).astype(np.uint32)
    else:
        a = (rng.integers(0, 4, n) << 20).astype(np.uint32)
    for bits in (32, 30):
        keys = dev(a, torch.int32)
        k.k_SimpleRadixSort(keys, n, key_bits=bits)
        assert u32(keys).tobytes() == np.sort(a).tobytes(), (pattern, bits)


# --------------------------------------------------------------- stage 3 --
@pytest.mark.parametrize("n", [1, 2, 5, 4095, 4096, 4097, 100_000, 1 << 21])
def test_unique_in_place(n):
    k = K()
    rng = np.random.default_rng(n)
    a = np.sort(rng.integers(0, max(n // 3, 1), n).astype(np.uint32))
    keys = dev(a, torch.int32)
    u = k.k_CountUnique(keys, n)
    ref_keys, ref_u = O.count_unique(a)
    assert u == ref_u
    assert u32(keys).tobytes() == ref_keys.tobytes()  # tail [U, n) keeps old values too


def test_unique_cfg1(golden):
    g = golden["cfg1_uniform_1m"]
    pts = O.init_random_vec4(g["n"])
    s = np.sort(O.morton(pts, 0.0, 1024.0))
    keys = dev(s, torch.int32)
    u = K().k_CountUnique(keys, g["n"])
    assert u == g["n_unique"]
    assert O.fnv1a64(u32(keys)[:u]) == g["hashes"]["sorted_unique"]
    assert O.fnv1a64(u32(keys)) == g["hashes"]["keys_after_unique"]


# ------------------------------------------------------------ stages 4-6 --
def _tree_on_gpu(codes: np.ndarray, nb: int):
    k = K()
    c = dev(codes, torch.int32)
    out = dict(prefix_n=garbage(nb, torch.uint8), has_leaf_left=garbage(nb, torch.uint8),
               has_leaf_right=garbage(nb, torch.uint8), left_child=garbage(nb, torch.int32),
               parent=garbage(nb, torch.int32))
    k.k_BuildRadixTree(nb, c, out["prefix_n"], out["has_leaf_left"], out["has_leaf_right"],
                       out["left_child"], out["parent"])
    return c, out


def test_radix_tree_edge_scan_small_cases(small_cases):
    k = K()
    for name, case in small_cases.items():
        codes = case["sorted_unique"]
        nb = len(codes) - 1
        c, t = _tree_on_gpu(codes, nb)
        for key in ["prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent"]:
            assert t[key][:nb].cpu().numpy().tobytes() == case[key].tobytes(), (name, key)
        ec = garbage(nb, torch.int32)
        k.k_EdgeCount(t["prefix_n"], t["parent"], ec, nb)
        assert ec[:nb].cpu().numpy().tobytes() == case["edge_count"].tobytes(), name
        ps = garbage(nb, torch.int32)
        assert k.k_PartialSum(ec, 0, nb, ps) == nb
        ps_h = ps[:nb].cpu().numpy().copy()
        ps_h[0] = 0  # the caller's ps[0] = 0 (apps/cpu_demo/main.cpp:118)
        assert ps_h.tobytes() == case["prefix_sum"].tobytes(), name
        assert k.octree_node_count(ec, ps, nb) == case["n_oct"]


@pytest.mark.parametrize("n", [1, 2, 4095, 4096, 4097, 1 << 20, (1 << 22) + 3])
def test_prefix_sum_random(n):
    rng = np.random.default_rng(n)
    a = rng.integers(-1000, 1000, n).astype(np.int32)
    out = garbage(n, torch.int32)
    K().k_PartialSum(dev(a), 0, n, out)
    assert out[:n].cpu().numpy().tobytes() == O.partial_sum(a).tobytes()


# ------------------------------------------------------------ stages 7-8 --
def test_octree_stages_small_cases(small_cases):
    k = K()
    for name, case in small_cases.items():
        codes = dev(case["sorted_unique"], torch.int32)
        nb = len(case["sorted_unique"]) - 1
        pn = dev(case["prefix_n"])
        hll = dev(case["has_leaf_left"])
        hlr = dev(case["has_leaf_right"])
        lc = dev(case["left_child"])
        par = dev(case["parent"])
        ec = dev(case["edge_count"])
        ps = dev(case["prefix_sum"])
        m = case["n_oct"]
        nodes = k.empty_oct_nodes(m)
        k.octree_root_init(nodes, codes, pn, 0.0, 1024.0)
        k.k_MakeOctNodes(nodes, ps, ec, codes, pn, par, 0.0, 1024.0, nb)
        k.k_LinkLeafNodes(nodes, ps, ec, codes, hll, hlr, pn, par, lc, nb)
        got = k.oct_nodes_to_numpy(nodes)
        if case["o7"]:
            expect = O.make_octree(case["sorted_unique"], {x: case[x] for x in
                                   ["prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent"]},
                                   case["edge_count"], case["prefix_sum"], 0.0, 1024.0)
        else:
            expect = case["oct_nodes"]
        assert got.tobytes() == expect.tobytes(), name


# ------------------------------------------------------------ whole build --
def _builder(n, cap=None):
    from pipeline_gb300.pipeline import OctreeBuilder

    return OctreeBuilder(n, cap)


def _compare_build(res, expect, name):
    assert (res["n_unique"], res["n_oct"]) == (expect["n_unique"], expect["n_oct"]), name
    assert res["status"] == 0, (name, res["status"])
    for key in STAGES:
        assert res[key].tobytes() == np.asarray(expect[key]).tobytes(), (name, key)


def test_build_small_cases(small_cases):
    for name, case in small_cases.items():
        n = len(case["points"])
        b = _builder(n)
        b.build(dev(case["points"]), 0.0, 1024.0)
        res = b.result()
        if case["o7"]:
            expect = O.build_all(case["points"], 0.0, 1024.0)
        else:
            expect = case
        _compare_build(res, expect, name)


@pytest.mark.parametrize("cfg", ["cfg1_uniform_1m", "cfg2_uniform_16m"])
def test_build_golden_hashes(golden, cfg):
    g = golden[cfg]
    from pipeline_gb300.kernels import k_InitRandomVec4

    pts = k_InitRandomVec4(None, g["n"], g["min"], g["range"], g["seed"])
    b = _builder(g["n"])
    b.build(dev(pts), g["min"], g["range"])
    res = b.result()
    assert (res["n_unique"], res["n_brt"], res["n_oct"], res["status"]) == \
        (g["n_unique"], g["n_brt"], g["n_oct"], 0)
    for key in STAGES:
        assert O.fnv1a64(res[key]) == g["hashes"][key], key


def _fuzz_cloud(rng, trial):
    n = int(rng.integers(3, 5000))
    kind = trial % 6
    if kind == 0:
        pts = rng.uniform(0, 1024, (n, 4))
    elif kind == 1:
        pts = rng.uniform(0, rng.uniform(1, 20), (n, 4))
    elif kind == 2:
        c = rng.uniform(0, 1024, (8, 3))
        s = rng.uniform(0.1, 30, (8, 3))
        idx = rng.integers(0, 8, n)
        pts = np.concatenate([rng.normal(c[idx], s[idx]), np.ones((n, 1))], 1)
        pts = np.clip(pts, 0, np.nextafter(np.float32(1024), np.float32(0)))
    elif kind == 3:
        pts = rng.uniform(0, 50, (n, 4))
        pts[0, :3] = 1023.5
    elif kind == 4:
        pts = rng.integers(0, 8, (n, 4)) * 1.0 + 0.5
    else:
        pts = rng.uniform(0, 50, (n, 4))
        pts[0, :3] = rng.uniform(0, 1024, 3)
        pts[1, :3] = rng.uniform(0, 1024, 3)
    pts = pts.astype(np.float32)
    pts[:, 3] = 1
    return pts


def test_build_fuzz_vs_oracle():
    rng = np.random.default_rng(2024)
    b = _builder(5000)
    for trial in range(240):
        pts = _fuzz_cloud(rng, trial)
        b.build(dev(pts), 0.0, 1024.0)
        res = b.result()
        expect = O.build_all(pts, 0.0, 1024.0)
        if expect["n_unique"] < 2:
            assert res["n_unique"] == expect["n_unique"]
            continue
        _compare_build(res, expect, f"trial{trial}")


def test_build_degenerate_sizes():
    b = _builder(16)
    for pts in [np.zeros((0, 4), np.float32), np.array([[1, 2, 3, 1]], np.float32),
                np.array([[1, 2, 3, 1]] * 5, np.float32),
                np.array([[1, 2, 3, 1], [700, 2, 3, 1]], np.float32)]:
        n = len(pts)
        b.build(dev(pts) if n else torch.empty((0, 4), device="cuda"), 0.0, 1024.0, n=n)
        c = b.counts()
        e = O.build_all(pts, 0.0, 1024.0) if n else {"n_unique": 0, "n_oct": 0}
        assert (c.n_unique, c.n_oct) == (e["n_unique"], e["n_oct"]), n
        if c.n_oct:
            assert b.result()["oct_nodes"].tobytes() == e["oct_nodes"].tobytes()


def test_build_unaligned_node_array():
    """OctNodes written to an array that is not 16-byte aligned (one node, 60
    bytes, into an allocation): finalize takes its vector-store path instead
    of the bulk copy, with the same bytes."""
    import ctypes as C

    from pipeline_gb300 import _lib

    pts = O.init_random_vec4(30000, 0.0, 1024.0, seed=21)
    expect = O.build_all(pts, 0.0, 1024.0)
    b = _builder(len(pts))
    shifted = torch.zeros((b.cap + 1, 15), dtype=torch.int32, device="cuda")
    out = _lib.OctBuildOutputs.from_buffer_copy(b._out)
    out.nodes = shifted.data_ptr() + 60  # 60 % 16 = 12
    rc = b.lib.oct_build_octree(C.c_void_p(dev(pts).data_ptr()), len(pts), 0.0, 1024.0,
                                C.byref(out), C.c_void_p(b.workspace.data_ptr()),
                                b.workspace.numel(), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "oct_build_octree")
    c = b.counts()
    assert (c.n_unique, c.n_oct, c.status) == (expect["n_unique"], expect["n_oct"], 0)
    got = shifted[1:1 + c.n_oct].cpu().numpy()
    assert got.tobytes() == expect["oct_nodes"].tobytes()


def test_build_capacity_status():
    from pipeline_gb300 import _lib

    pts = O.init_random_vec4(20000)
    b = _builder(20000, cap=100)
    b.build(dev(pts), 0.0, 1024.0)
    c = b.counts()
    assert c.status & _lib.OCT_STATUS_CAPACITY
    assert c.n_oct == O.build_all(pts, 0.0, 1024.0)["n_oct"]


def test_graph_replay_is_deterministic(golden):
    g = golden["cfg1_uniform_1m"]
    pts = dev(O.init_random_vec4(g["n"]))
    b = _builder(g["n"])
    b.capture(pts, 0.0, 1024.0)
    for _ in range(3):
        b.nodes.fill_(-1)
        b.replay()
        res = b.result()
        assert O.fnv1a64(res["oct_nodes"]) == g["hashes"]["oct_nodes"]
        assert O.fnv1a64(res["parent"]) == g["hashes"]["parent"]
