"""Pins the CPU oracle (oracle/oracle.c) to the reference's own outputs.

The fixtures in tests/golden/ were produced by running the reference's
unmodified CPU stage functions (tests/golden/make_golden.py). Stage 8 of a case
marked "o7" is not reference output (the reference never returns there); the
oracle's contract value is checked against its own stage-7 prefix instead.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

STAGES = ["morton", "sorted_unique", "keys_after_unique", "prefix_n", "has_leaf_left",
          "has_leaf_right", "left_child", "parent", "edge_count", "prefix_sum", "oct_nodes"]


def test_kat_sort(golden):
    """tests/xmake.lua:9-13: "10 9 ... 1" sorts to "1 2 ... 10"."""
    kat = golden["kat_sort"]
    for threads in (1, 4):
        out = O.radix_sort(np.array(kat["input"], np.uint32), threads=threads)
        assert out.tolist() == kat["expected"]


def test_generator_first_points(golden):
    pts = O.init_random_vec4(4)
    assert pts.tolist() == golden["cfg1_uniform_1m"]["first_points"]


@pytest.mark.parametrize("name", ["uniform_1000", "uniform_4097", "tinybox_3000", "clusters_2500",
                                  "outlier_1500", "grid_2000", "three_points", "top_edge_64"])
def test_small_cases_bytes(small_cases, name):
    case = small_cases[name]
    o = O.build_all(case["points"], 0.0, 1024.0)
    assert o["n_unique"] == case["n_unique"]
    assert o["n_oct"] == case["n_oct"]
    for k in STAGES:
        if k == "oct_nodes" and case["o7"]:
            continue
        assert o[k].tobytes() == case[k].tobytes(), k


def test_cfg1_hashes(golden):
    g = golden["cfg1_uniform_1m"]
    pts = O.init_random_vec4(g["n"], g["min"], g["range"], g["seed"])
    assert O.fnv1a64(pts) == g["input_hash"]
    o = O.build_all(pts, g["min"], g["range"])
    assert (o["n_unique"], o["n_oct"]) == (g["n_unique"], g["n_oct"])
    for k, h in g["hashes"].items():
        assert O.fnv1a64(o[k]) == h, k


@pytest.mark.slow
def test_cfg2_hashes(golden):
    g = golden["cfg2_uniform_16m"]
    pts = O.init_random_vec4(g["n"], g["min"], g["range"], g["seed"])
    o = O.build_all(pts, g["min"], g["range"], threads=4)
    assert (o["n_unique"], o["n_oct"]) == (g["n_unique"], g["n_oct"])
    for k, h in g["hashes"].items():
        assert O.fnv1a64(o[k]) == h, k


def test_per_stage_functions_match_build_all(small_cases):
    case = small_cases["clusters_2500"]
    pts = case["points"]
    m = O.morton(pts, 0.0, 1024.0)
    s = O.radix_sort(m)
    k, u = O.count_unique(s)
    tree = O.build_radix_tree(k, u - 1)
    ec = O.edge_count(tree["prefix_n"], tree["parent"])
    ps = O.partial_sum(ec)
    ps[0] = 0
    nodes = O.make_octree(k, tree, ec, ps, 0.0, 1024.0)
    assert nodes.tobytes() == case["oct_nodes"].tobytes()


def test_parallel_stages_match_sequential_where_deterministic(small_cases):
    """Stages 1-6 are deterministic under threads; the octree stage is not (a
    race in the reference), so only it is excluded."""
    case = small_cases["uniform_4097"]
    a = O.build_all(case["points"], 0.0, 1024.0, threads=1)
    b = O.build_all(case["points"], 0.0, 1024.0, threads=4, parallel_octree=True)
    for k in STAGES[:-1]:
        assert a[k].tobytes() == b[k].tobytes(), k


def test_o7_detector():
    """three_points reaches radix node 0 in a LinkLeaf walk (contract O7)."""
    pts = np.array([[1, 2, 3, 1], [900, 10, 20, 1], [512, 512, 512, 1]], np.float32)
    o = O.build_all(pts, 0.0, 1024.0)
    assert O.o7_walks(o["edge_count"], o["has_leaf_left"], o["has_leaf_right"], o["parent"]) > 0


def test_planted_mistake_is_caught(small_cases):
    """A wrong oracle value must fail the byte comparison (the check has teeth)."""
    case = small_cases["uniform_1000"]
    o = O.build_all(case["points"], 0.0, 1024.0)
    bad = o["prefix_sum"].copy()
    bad[len(bad) // 2] += 1
    assert bad.tobytes() != case["prefix_sum"].tobytes()


def test_device_generator_restatement_matches_numpy():
    """The oracle's copy of the reference's device generator against an
    independent numpy statement of the same integer steps (min = 0 and a
    power-of-two range make the fused multiply-add exact in float64)."""
    n, seed, rg = 3000, 114514, 1024.0
    i = np.arange(n, dtype=np.uint64)
    m32 = np.uint64(0xFFFFFFFF)
    b = (i << np.uint64(2)) & m32
    sd = np.uint64(seed & 0xFFFFFFFF)
    z1, z2, z3, z4 = [((b + np.uint64(k)) * sd) & m32 for k in range(4)]
    z1 = ((((z1 & np.uint64(4294967294)) << np.uint64(12)) & m32) ^ ((((z1 << np.uint64(13)) & m32) ^ z1) >> np.uint64(19)))
    z2 = ((((z2 & np.uint64(4294967288)) << np.uint64(4)) & m32) ^ ((((z2 << np.uint64(2)) & m32) ^ z2) >> np.uint64(25)))
    z3 = ((((z3 & np.uint64(4294967280)) << np.uint64(17)) & m32) ^ ((((z3 << np.uint64(3)) & m32) ^ z3) >> np.uint64(11)))
    z4 = (z4 * np.uint64(1664525) + np.uint64(1013904223)) & m32
    vals = [z1 ^ z2, z2 ^ z3, z3 ^ z4, z1 ^ z4]
    want = np.stack([((v & np.uint64(0xFFFFFF)).astype(np.float64) / 16777216.0 * rg).astype(np.float32)
                     for v in vals], 1)
    got = O.init_random_vec4_gpu(n, 0.0, rg, seed)
    assert got.tobytes() == want.tobytes()


def test_check_tree_restatement_small():
    """checkTree counts on a hand-made three-node octree."""
    nodes = np.zeros(3, O.OCTNODE_DTYPE)
    nodes[0]["child_node_mask"] = 0b101
    nodes[0]["children"][0] = 1
    nodes[0]["children"][2] = 2
    nodes[1]["child_leaf_mask"] = 0b10   # child 1 of prefix 0: keys 0b000001...
    nodes[1]["children"][1] = 0
    nodes[2]["child_leaf_mask"] = 0b1    # child 0 of prefix 2: key 0b010000... expected
    nodes[2]["children"][0] = 1
    codes = np.array([1 << 24, 5 << 24], np.uint32)  # top 6 bits 000001 and 000101
    # code 0 sits under prefix 0b000001 (match); code 1 under 0b000101, checked against 0b010000
    assert O.check_tree(nodes, codes, 0, 0) == (3, 2, 1, 0)
    nodes[2]["child_node_mask"] = 0b1000000
    nodes[2]["children"][6] = 9  # out of range
    assert O.check_tree(nodes, codes, 0, 0) == (3, 2, 1, 1)


def test_init_sequences_match_reference():
    """k_InitDescending / k_InitAscending (kernels/00_init.cpp:5-17): the
    reference's own functions, where they are built here, give n - i and i."""
    ref = O.load_ref()
    if ref is None:
        pytest.skip("the reference's CPU kernels are not built here")
    for n in (0, 1, 10, 100_003):
        d = np.full(max(n, 1), 0xDEADBEEF, np.uint32)
        a = d.copy()
        ref.ref_init_descending(d.ctypes.data, n)
        ref.ref_init_ascending(a.ctypes.data, n)
        assert d[:n].tolist() == (n - np.arange(n)).tolist()
        assert a[:n].tolist() == np.arange(n).tolist()


def _device_init_fixture():
    path = os.path.join(os.path.dirname(__file__), "golden", "device_init.json")
    if not os.path.exists(path):
        return []
    with open(path) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", _device_init_fixture(),
                         ids=lambda c: f'n{c["n"]}_seed{c["seed"]}')
def test_device_generator_restatement_matches_reference_gpu_output(case):
    """The oracle's restatement of gpu::k_InitRandomVec4 against the values the
    reference's own kernel (kernels/cuda/00_init.cu, run on a GB300 as its
    driver launches it) produced: tests/golden/device_init.json."""
    got = O.init_random_vec4_gpu(case["n"], case["min"], case["range"], case["seed"])
    assert got[:2].tolist() == case["first_points"][:case["n"]]
    assert O.fnv1a64(got) == case["hash"]
