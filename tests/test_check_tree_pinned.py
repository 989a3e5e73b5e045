"""checkTree pinned to the reference's own checkTree (apps/cpu_demo/main.cpp:13-35).

tests/golden/check_tree.json holds, for the octrees of
tests/golden/check_tree_cases.py, how many "oh no..." lines the reference's
checkTree printed (compiled unmodified from the demo; see
tests/golden/make_check_tree.py). The oracle's restatement and the GPU's
oct_check_tree must count the same mismatches on the same octrees.
"""
import json
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import check_tree_cases as CT  # noqa: E402

with open(os.path.join(HERE, "golden", "check_tree.json")) as _f:
    FIXTURE = json.load(_f)["cases"]

_built = {}


def _octree(case):
    key = (case["name"], case["n"], case["low"], case["width"], case["seed"])
    if key not in _built:
        pts = CT.cloud(case["n"], case["low"], case["width"], case["seed"])
        _built[key] = O.build_all(pts, 0.0, 1024.0, threads=8)
    b = _built[key]
    codes = b["sorted_unique"]
    prefix, code_len = CT.root_of(b)
    assert (prefix, code_len) == (case["root_prefix"], case["root_code_len"])
    nodes = CT.form(b["oct_nodes"], len(codes), code_len, case["form"])
    assert O.fnv1a64(nodes) == case["nodes_hash"], "not the octree the reference checked"
    return nodes, codes, prefix, code_len


def test_fixture_covers_every_case_and_form():
    seen = {(c["name"], c["form"]) for c in FIXTURE}
    assert seen == {(name, f) for name, *_ in CT.CASES for f in CT.FORMS}
    assert any(c["reference_oh_no"] > 1000 for c in FIXTURE)


@pytest.mark.parametrize("case", FIXTURE, ids=lambda c: f'{c["name"]}-{c["form"]}')
def test_oracle_check_tree_matches_reference(case):
    nodes, codes, prefix, code_len = _octree(case)
    got = O.check_tree(nodes, codes, prefix, code_len)
    assert got[2] == case["reference_oh_no"]
    assert got[3] == 0
    assert list(got) == case["oracle_counts"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", FIXTURE, ids=lambda c: f'{c["name"]}-{c["form"]}')
def test_gpu_check_tree_matches_reference(case):
    import torch

    from pipeline_gb300.kernels import check_tree

    nodes, codes, prefix, code_len = _octree(case)
    d_nodes = torch.from_numpy(nodes.view(np.int32).reshape(-1, 15).copy()).cuda()
    d_codes = torch.from_numpy(codes.view(np.int32).copy()).cuda()
    got = check_tree(d_nodes, len(nodes), d_codes, len(codes), prefix, code_len)
    assert got[2] == case["reference_oh_no"]
    assert list(got) == case["oracle_counts"]
