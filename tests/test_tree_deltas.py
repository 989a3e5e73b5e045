"""CPU check of the radix-tree restatement the delta-based kernels use
(csrc/tree_tiled.cu) against the oracle's k_BuildRadixTree and k_EdgeCount.

For strictly increasing codes the tree is the Cartesian tree of the adjacent
deltas D[q] = delta(codes[q], codes[q + 1]): the node split at q covers
[a + 1, b] (a, b the nearest positions with a smaller delta), has index a + 1
when D[a] > D[b] and b otherwise, and its edge count is
D[q]/3 - max(D[a], D[b])/3; only radix node 0 follows the reference's own
convention (range [0, n - 1]). This statement is written here in plain
Python, position by position, and compared with the oracle on code sets that
cover both root forms.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _delta(a: int, b: int) -> int:
    x = (a ^ b) & 0xFFFFFFFF
    clz = 32 if x == 0 else 32 - x.bit_length()
    return (clz - 1) & 0xFF


def tree_from_deltas(codes):
    n = len(codes) - 1
    d = [min(_delta(int(codes[q]), int(codes[q + 1])), 31) for q in range(n)]
    a = [-1] * n
    b = [n] * n
    st = []
    for q in range(n):  # nearest smaller to the left
        while st and d[st[-1]] >= d[q]:
            st.pop()
        a[q] = st[-1] if st else -1
        st.append(q)
    st = []
    for q in range(n - 1, -1, -1):  # nearest smaller to the right
        while st and d[st[-1]] >= d[q]:
            st.pop()
        b[q] = st[-1] if st else n
        st.append(q)
    pn = np.zeros(n, np.uint8)
    hll = np.zeros(n, np.uint8)
    hlr = np.zeros(n, np.uint8)
    lc = np.zeros(n, np.int32)
    par = np.full(n, -7, np.int32)  # -7: never written
    ec = np.zeros(n, np.int32)

    def root(q, x, short):
        ll, lr = q == 0, q + 1 == n - 1
        pn[0], lc[0], hll[0], hlr[0], par[0] = x, q, ll, lr, 0
        if short or lr:
            par[n - 1] = 0
        if not short:
            if not ll:
                par[q] = 0
            if not lr and q + 1 < n:
                par[q + 1] = 0

    for q in range(n):
        x, aa, bb = d[q], a[q], b[q]
        da = -1 if aa < 0 else d[aa]
        db = -1 if bb >= n else d[bb]
        if aa < 0 and bb >= n:
            if q <= n - 2:
                root(q, x, False)
            continue
        i = bb if aa < 0 else (aa + 1 if bb >= n else (aa + 1 if da > db else bb))
        ll, lr = aa + 1 == q, bb == q + 1
        short = aa < 0 and bb == n - 1
        pn[i], lc[i], hll[i], hlr[i] = x, q, ll, lr
        if not ll:
            par[q] = i
        if not lr:
            par[q + 1] = i
        ec[i] = 0 if short else x // 3 - max(da, db) // 3
        if short:
            root(q, x, True)
    return dict(prefix_n=pn, has_leaf_left=hll, has_leaf_right=hlr, left_child=lc, parent=par), ec


def _codes(kind, n_codes, rng):
    if kind == "uniform":
        c = np.unique(rng.integers(0, 1 << 30, n_codes + 16))[:n_codes]
    elif kind == "consecutive":
        c = np.arange(n_codes) + int(rng.integers(0, 1000))
    elif kind == "clustered":
        base = rng.integers(0, 1 << 30, 4)
        c = np.unique(np.concatenate([b + rng.integers(0, 64 + 2 * n_codes, n_codes) for b in base])
                      % (1 << 30))[:n_codes]
    elif kind == "short_root":  # the smallest delta at n - 1
        c = np.append(np.unique(rng.integers(0, 1 << 12, n_codes + 64))[:n_codes - 1], (1 << 29) + 5)
    elif kind == "low_outlier":  # the smallest delta at 0
        c = np.insert(np.unique(rng.integers(1 << 29, (1 << 29) + (1 << 12), n_codes + 64))
                      [:n_codes - 1], 0, 3)
    else:  # "two_high": the smallest delta at n - 2
        c = np.append(np.unique(rng.integers(0, 1 << 20, n_codes + 64))[:max(n_codes - 2, 0)],
                      [(1 << 29) + 1, (1 << 29) + 2])[-n_codes:]
    c = np.unique(np.asarray(c, np.int64)).astype(np.uint32)
    return c


@pytest.mark.parametrize("kind", ["uniform", "consecutive", "clustered", "short_root",
                                  "low_outlier", "two_high"])
def test_cartesian_tree_matches_oracle(kind):
    rng = np.random.default_rng(len(kind))
    for n_codes in list(range(2, 34)) + [100, 257, 1500]:
        codes = _codes(kind, n_codes, rng)
        if len(codes) < 2:
            continue
        n = len(codes) - 1
        if n == 1:  # a single node: the kernels run the reference's search steps
            continue
        ref = O.build_radix_tree(codes, n)
        got, ec = tree_from_deltas(codes)
        for key in ["prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent"]:
            assert np.array_equal(np.asarray(ref[key]).astype(np.int64),
                                  got[key].astype(np.int64)), (kind, n_codes, key)
        assert np.array_equal(O.edge_count(ref["prefix_n"], ref["parent"]), ec), (kind, n_codes)
