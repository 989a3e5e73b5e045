"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Run in a container that has the reference sources (it builds oracle/_ref/ with
oracle/build_ref.sh and calls the reference's CPU stage functions through
oracle/ref_harness.cpp). Writes:

  golden.json       known-answer test of tests/xmake.lua:9-13, plus for the
                    1,048,576- and 16,777,216-point uniform clouds (seed 114514,
                    [0,1024)^3) the first input points, U, M and FNV-1a-64
                    hashes of every stage buffer;
  small_cases.npz   complete inputs and stage outputs of small clouds (uniform,
                    tiny-box duplicates, Gaussian clusters, far outliers, grid
                    points) for byte-for-byte comparisons.

Every value comes from the reference implementation, called in the order of
apps/cpu_demo/main.cpp:72-154 with the oracle contract (radix tree over U-1
nodes, zeroed outputs, 1-thread octree stages). Where a LinkLeaf walk would
reach radix node 0 (the reference then never returns), the case records
"o7": true and its oct_nodes come from stage 7 only plus the oracle's
contract for stage 8; the test then checks stage 8 against the oracle.

Usage: python tests/golden/make_golden.py [--skip-16m]
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

STAGE_KEYS = ["morton", "sorted_unique", "keys_after_unique", "prefix_n", "has_leaf_left",
              "has_leaf_right", "left_child", "parent", "edge_count", "prefix_sum", "oct_nodes"]


def _p(a):
    return a.ctypes.data


def reference_pipeline(ref, pts: np.ndarray, mn: float, rg: float) -> dict:
    n = len(pts)
    ref.ref_set_threads(1)
    keys = np.empty(max(n, 1), np.uint32)
    ref.ref_morton(_p(pts), _p(keys), n, mn, rg)
    morton = keys[:n].copy()
    ref.ref_radix_sort(_p(keys), n)
    U = ref.ref_count_unique(_p(keys), n)
    B = U - 1
    pad = 8  # the reference writes parent[1] for a one-node tree
    prefix = np.zeros(B + pad, np.uint8)
    hll = np.zeros(B + pad, np.uint8)
    hlr = np.zeros(B + pad, np.uint8)
    left = np.zeros(B + pad, np.int32)
    parent = np.zeros(B + pad, np.int32)
    ref.ref_build_radix_tree(B, _p(keys), _p(prefix), _p(hll), _p(hlr), _p(left), _p(parent))
    ec = np.zeros(B + pad, np.int32)
    ref.ref_edge_count(_p(prefix), _p(parent), _p(ec), B)
    ps = np.zeros(B + pad, np.int32)
    ref.ref_partial_sum(_p(ec), 0, B, _p(ps))
    ps[0] = 0
    M = O.oct_node_count(ec[:B], ps[:B])
    nodes = np.zeros(M + 64, O.OCTNODE_DTYPE)
    ref.ref_root_init(_p(nodes), _p(keys), _p(prefix), mn, rg)
    ref.ref_make_oct_nodes(_p(nodes), _p(ps), _p(ec), _p(keys), _p(prefix), _p(parent), mn, rg, B)
    o7 = O.o7_walks(ec[:B], hll[:B], hlr[:B], parent[:B]) > 0
    if not o7:
        ref.ref_link_leaf_nodes(_p(nodes), _p(ps), _p(ec), _p(keys), _p(hll), _p(hlr), _p(prefix),
                                _p(parent), _p(left), B)
    assert not nodes[M:].tobytes().strip(b"\0"), "reference wrote past M"
    return dict(n_unique=U, n_oct=M, o7=bool(o7), morton=morton, sorted_unique=keys[:U].copy(),
                keys_after_unique=keys[:n].copy(), prefix_n=prefix[:B].copy(),
                has_leaf_left=hll[:B].copy(), has_leaf_right=hlr[:B].copy(),
                left_child=left[:B].copy(), parent=parent[:B].copy(), edge_count=ec[:B].copy(),
                prefix_sum=ps[:B].copy(), oct_nodes=nodes[:M].copy())


def small_inputs():
    rng = np.random.default_rng(20241203)
    cases = []

    def add(name, pts):
        pts = np.asarray(pts, np.float32).copy()
        pts[:, 3] = 1.0
        cases.append((name, pts))

    add("uniform_1000", rng.uniform(0, 1024, (1000, 4)))
    add("uniform_4097", rng.uniform(0, 1024, (4097, 4)))
    add("tinybox_3000", rng.uniform(0, 6, (3000, 4)))
    c = rng.uniform(0, 1024, (8, 3))
    s = rng.uniform(0.2, 25, (8, 3))
    idx = rng.integers(0, 8, 2500)
    g = np.clip(rng.normal(c[idx], s[idx]), 0, np.nextafter(np.float32(1024), np.float32(0)))
    add("clusters_2500", np.concatenate([g, np.ones((2500, 1))], 1))
    o = rng.uniform(0, 40, (1500, 4))
    o[0, :3] = 1023.5
    add("outlier_1500", o)
    add("grid_2000", rng.integers(0, 16, (2000, 4)) * 1.0 + 0.25)
    add("three_points", [[1, 2, 3, 1], [900, 10, 20, 1], [512, 512, 512, 1]])
    add("top_edge_64", np.concatenate([np.full((64, 3), 1024.0), np.ones((64, 1))], 1) -
        np.concatenate([rng.uniform(0, 3, (64, 3)), np.zeros((64, 1))], 1))
    return cases


def main(argv):
    ref_path = O.build_ref()
    if ref_path is None:
        raise SystemExit("reference sources are not available here")
    ref = O.load_ref()
    out = {"generator": "tests/golden/make_golden.py", "hash": "fnv1a64 over raw little-endian buffers",
           "kat_sort": {"source": "tests/xmake.lua:9-13, tests/test_simple_radix_sort_cpu.cpp:16-19"}}

    kat = np.array([10, 9, 8, 7, 6, 5, 4, 3, 2, 1], np.uint32)
    ref.ref_set_threads(4)
    ref.ref_radix_sort(_p(kat), len(kat))
    out["kat_sort"].update(input=[10, 9, 8, 7, 6, 5, 4, 3, 2, 1], expected=[int(v) for v in kat])

    sizes = [("cfg1_uniform_1m", 1 << 20)]
    if "--skip-16m" not in argv:
        sizes.append(("cfg2_uniform_16m", 1 << 24))
    for name, n in sizes:
        pts = np.empty((n, 4), np.float32)
        ref.ref_init_random_vec4(_p(pts), n, 0.0, 1024.0, 114514)
        r = reference_pipeline(ref, pts, 0.0, 1024.0)
        out[name] = {
            "n": n, "min": 0.0, "range": 1024.0, "seed": 114514,
            "first_points": pts[:4].tolist(), "input_hash": O.fnv1a64(pts),
            "n_unique": r["n_unique"], "n_brt": r["n_unique"] - 1, "n_oct": r["n_oct"], "o7": r["o7"],
            "hashes": {k: O.fnv1a64(r[k]) for k in STAGE_KEYS},
        }
        print(name, out[name]["n_unique"], out[name]["n_oct"], out[name]["o7"])

    arrays = {}
    meta = []
    for name, pts in small_inputs():
        r = reference_pipeline(ref, pts, 0.0, 1024.0)
        meta.append({"name": name, "n": len(pts), "n_unique": r["n_unique"], "n_oct": r["n_oct"],
                     "o7": r["o7"]})
        arrays[f"{name}__points"] = pts
        for k in STAGE_KEYS:
            arrays[f"{name}__{k}"] = r[k]
        print(name, meta[-1])
    out["small_cases"] = meta
    np.savez_compressed(os.path.join(HERE, "small_cases.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:])
