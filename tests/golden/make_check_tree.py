"""Generate tests/golden/check_tree.json from the reference's own checkTree.

Run where the reference sources are (oracle/build_ref.sh builds
oracle/_ref/ref_check from the unmodified apps/cpu_demo/main.cpp). For every
octree of tests/golden/check_tree_cases.py (built by the oracle, which is
pinned to the reference's stage outputs by tests/golden/golden.json) and each
of its three forms, it runs the reference's checkTree
(apps/cpu_demo/main.cpp:13-35) from the root and records how many
"oh no..." lines it printed, with the FNV-1a-64 of the checked node array and
the oracle's own counts (visited, leaf checks, mismatches, rejected).

Usage: python tests/golden/make_check_tree.py
"""
from __future__ import annotations

import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402

import check_tree_cases as CT  # noqa: E402


def reference_oh_no(nodes: np.ndarray, codes: np.ndarray, prefix: int, code_len: int) -> int:
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_check")
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
        f.write(struct.pack("<i", len(nodes)))
        f.write(np.ascontiguousarray(nodes, O.OCTNODE_DTYPE).tobytes())
        f.write(struct.pack("<i", len(codes)))
        f.write(np.ascontiguousarray(codes, np.uint32).tobytes())
        f.write(struct.pack("<Iii", prefix, code_len, 0))
        path = f.name
    try:
        r = subprocess.run([exe, path], stdout=subprocess.PIPE, check=True, timeout=600)
    finally:
        os.unlink(path)
    lines = r.stdout.decode().splitlines()
    assert all(line == "oh no..." for line in lines), lines[:3]
    return len(lines)


def main() -> None:
    if O.build_ref() is None or not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "ref_check")):
        raise SystemExit("reference sources are not available here")
    out = {"generator": "tests/golden/make_check_tree.py",
           "source": "apps/cpu_demo/main.cpp:13-35 (checkTree), run unmodified",
           "cases": []}
    for name, n, low, width, seed in CT.CASES:
        built = O.build_all(CT.cloud(n, low, width, seed), 0.0, 1024.0, threads=8)
        codes = built["sorted_unique"]
        prefix, code_len = CT.root_of(built)
        for which in CT.FORMS:
            nodes = CT.form(built["oct_nodes"], len(codes), code_len, which)
            counts = O.check_tree(nodes, codes, prefix, code_len)
            assert counts[3] == 0, (name, which, counts)  # every step in range: recursion ends
            oh_no = reference_oh_no(nodes, codes, prefix, code_len)
            out["cases"].append({"name": name, "form": which, "n": n, "low": low, "width": width,
                                 "seed": seed, "n_oct": len(nodes), "nodes_hash": O.fnv1a64(nodes),
                                 "root_prefix": prefix, "root_code_len": code_len,
                                 "reference_oh_no": oh_no, "oracle_counts": list(counts)})
            print(name, which, oh_no, counts)
    with open(os.path.join(HERE, "check_tree.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
