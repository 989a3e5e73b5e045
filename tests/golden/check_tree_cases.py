"""Octrees on which checkTree (apps/cpu_demo/main.cpp:13-35) is pinned.

Shared by tests/golden/make_check_tree.py (which runs the reference's own
checkTree on them and records what it prints) and by the tests (which rebuild
the same octrees and compare the oracle's and the GPU's counts with it).

checkTree follows child_node_mask bits without bounds checks. On the
reference's own octrees some of those bits lead out of the node array or past
30 code bits (the overlapping slot ranges of the inclusive prefix sum let
leaf links and node links share a child slot), where checkTree reads out of
bounds or recurses without end. So each octree is first made safe: every
mask bit that the traversal would follow out of the arrays or past 30 bits
is cleared, repeated until none is left (the traversal then ends and stays
in bounds). The reference's builds also leave child_leaf_mask at 0 (SetLeaf
clears the bit, include/shared/oct.h:16-21), which would leave the leaf
comparison unexercised, so each safe octree is checked in three forms:

  built    the safe octree (leaf masks 0);
  leaves   leaf-mask bits set where the child slot was written but its
           node-mask bit is clear (the linked leaves, except a link to
           leaf 0, which looks unwritten), then made safe again;
  planted  `leaves`, then on every 5th node with leaf bits its lowest leaf
           child moved to the next code index (a wrong leaf, usually).

All three are deterministic functions of the built octree.
"""
from __future__ import annotations

import numpy as np

# (name, n, low, width, seed): clouds drawn by the reference's generator
# (k_InitRandomVec4, restated by the oracle and pinned to the reference), in
# [low, low + width)^3 and quantised over [0, 1024)^3: a small uniform cloud,
# a cloud in a 24-unit box (duplicates, deep chains) and the 1,048,576-point
# uniform cloud.
CASES = [
    ("uniform_5000", 5000, 0.0, 1024.0, 3),
    ("smallbox_20000", 20000, 500.0, 24.0, 4),
    ("uniform_1m", 1 << 20, 0.0, 1024.0, 114514),
]
FORMS = ("built", "leaves", "planted")


def cloud(n: int, low: float, width: float, seed: int) -> np.ndarray:
    from oracle import oracle as O

    return O.init_random_vec4(n, low, width, seed)


def root_of(built: dict) -> tuple[int, int]:
    """(prefix, code_len) of the root, as apps/cpu_demo/main.cpp:125-128 sets it up."""
    codes = built["sorted_unique"]
    level = int(built["prefix_n"][0]) // 3 if len(built["prefix_n"]) else 0
    return int(codes[0]) >> (30 - 3 * level), 3 * level


BITS = (1 << np.arange(8)).astype(np.int32)


def _unsafe_bits(nodes: np.ndarray, n_codes: int, code_len: int):
    """Per node, the node-mask and leaf-mask bits whose step checkTree would
    take out of the arrays or past 30 bits, found by walking every path from
    the root level by level (as checkTree's recursion does)."""
    n = len(nodes)
    kids = nodes["children"]
    nmask = nodes["child_node_mask"]
    lmask = nodes["child_leaf_mask"]
    bad_n = np.zeros(n, np.int32)
    bad_l = np.zeros(n, np.int32)
    front = np.array([0], np.int64)
    length = code_len
    while len(front):
        deep = length + 3 > 30
        nxt = []
        for c in range(8):
            take = (nmask[front] & BITS[c]) != 0
            ch = kids[front, c]
            out = take & ((ch < 0) | (ch >= n) | deep)
            np.bitwise_or.at(bad_n, front[out], BITS[c])
            nxt.append(ch[take & ~out].astype(np.int64))
            leaf = (lmask[front] & BITS[c]) != 0
            lout = leaf & ((ch < 0) | (ch >= n_codes) | deep)
            np.bitwise_or.at(bad_l, front[lout], BITS[c])
        front = np.concatenate(nxt)
        length += 3
    return bad_n, bad_l


def make_safe(nodes: np.ndarray, n_codes: int, code_len: int) -> np.ndarray:
    out = nodes.copy()
    while True:
        bad_n, bad_l = _unsafe_bits(out, n_codes, code_len)
        if not bad_n.any() and not bad_l.any():
            return out
        out["child_node_mask"] &= ~bad_n
        out["child_leaf_mask"] &= ~bad_l


def form(nodes: np.ndarray, n_codes: int, code_len: int, which: str) -> np.ndarray:
    out = make_safe(nodes, n_codes, code_len)
    if which == "built":
        return out
    kids = out["children"]
    nmask = out["child_node_mask"]
    leaf = (kids != 0) & ((nmask[:, None] & BITS[None, :]) == 0)
    out["child_leaf_mask"] = (leaf * BITS[None, :]).sum(1).astype(np.int32)
    out = make_safe(out, n_codes, code_len)
    if which == "leaves":
        return out
    assert which == "planted"
    kids = out["children"]
    has = np.nonzero(out["child_leaf_mask"])[0][::5]
    for p in has:
        c = int(np.nonzero(out["child_leaf_mask"][p] & BITS)[0][0])
        kids[p, c] = (kids[p, c] + 1) % n_codes
    return out
