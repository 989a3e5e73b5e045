"""Pins the CPU oracle (oracle/oracle.c) to the reference's own outputs.

The fixtures in tests/golden/ were produced by running the reference's
unmodified CPU stage functions (tests/golden/make_golden.py). Stage 8 of a case
marked "o7" is not reference output (the reference never returns there); the
oracle's contract value is checked against its own stage-7 prefix instead.
"""
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
