// Karras radix-tree node construction shared by the single-cloud and the
// batched builds.
#pragma once

#include "kernels.cuh"

namespace octgb {

// --------------------------------------------------------------------------
// Karras radix tree (stage 4), one thread per node.
// Replaces k_BuildRadixTree (include/kernels/04_radix_tree.hpp:5-11,
// kernels/04_radix_tree.cpp:39-121). The search steps are the reference's,
// step for step, since its root convention (d = 1, l = n - 1) and cut-offs
// show in the output.
//
// Parent writes: only radix nodes 0 and n-1 can claim the same children, and
// only when the root, which spans keys [0, n-1], has a longer common prefix
// than keys [0, n] ("short root"); then node n-1 spans the same range, makes
// the same split and, being later, wins. Node 0 therefore skips its parent
// writes in that case. Entries nobody writes are parent[0] and, when the
// root is short or its right child is the leaf n-1, parent[n-1]; node 0
// zeroes exactly those, so no pre-clear of parent[] is needed.
// --------------------------------------------------------------------------
// Code reads go through an accessor (GlobalCodes: codes[] in global memory).
struct GlobalCodes {
  const uint32_t* __restrict__ g;
  __device__ __forceinline__ uint32_t operator[](int j) const { return g[j]; }
};

// Index arithmetic is 32-bit: n <= OCT_MAX_N < 2^30, so an in-range step lmax
// is at most 2^29, the first out-of-range one at most 2^30, and every sum
// below stays under 2^31. The reference's divisions by powers of two 2^k are
// shifts (identical for these non-negative operands): t = lmax / 2^k and
// t = ceil(l / 2^k).
template <class Codes>
__device__ __forceinline__ void radix_node(int i, int n, const Codes& codes,
                                           uint8_t* __restrict__ prefix_n,
                                           uint8_t* __restrict__ hll, uint8_t* __restrict__ hlr,
                                           int* __restrict__ left_child,
                                           int* __restrict__ parent) {
  const uint32_t ci = codes[i];
  int d, l = 0;
  if (i == 0) {
    d = 1;
    l = n - 1;
  } else {
    const int diff = delta_u8(ci, codes[i + 1]) - delta_u8(ci, codes[i - 1]);
    d = (diff > 0) - (diff < 0);
    const int dmin = delta_u8(ci, codes[i - d]);
    int lmax = 2;
    while (true) {
      const int e = i + lmax * d;
      if (e < 0 || e > n || delta_u8(ci, codes[e]) <= dmin) break;
      lmax <<= 1;
    }
    const int lcut = (d == -1) ? i : n - i;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
      if (l + t <= lcut && delta_u8(ci, codes[i + (l + t) * d]) > dmin) l += t;
  }
  const int j = i + l * d;
  const int dnode = delta_u8(ci, codes[j]);
  prefix_n[i] = (uint8_t)dnode;
  int s = 0;
  if (l > 0) {
    const int lg = log2_ceil_u32((uint32_t)l);
    const int scut = (d == -1) ? i - 1 : n - i - 1;
    for (int k = 1; k <= lg; ++k) {
      const int t = (l + (1 << k) - 1) >> k;
      if (s + t <= scut && delta_u8(ci, codes[i + (s + t) * d]) > dnode) s += t;
    }
  }
  const int gamma = i + s * d + min(d, 0);
  left_child[i] = gamma;
  const bool leaf_l = min(i, j) == gamma;
  const bool leaf_r = max(i, j) == gamma + 1;
  hll[i] = leaf_l;
  hlr[i] = leaf_r;
  if (i == 0) {
    parent[0] = 0;
    const bool short_root = n >= 2 && delta_u8(ci, codes[n - 1]) > delta_u8(ci, codes[n]);
    if (n >= 2 && (short_root || leaf_r)) parent[n - 1] = 0;
    if (short_root) return;
  }
  if (!leaf_l && gamma < n) parent[gamma] = i;
  if (!leaf_r && gamma + 1 < n) parent[gamma + 1] = i;
}

// --------------------------------------------------------------------------
// Bottom-up construction of the same tree (stage 4) plus the edge counts of
// stage 5, for the whole-build paths.
//
// Leaves are the U = N codes, radix nodes the N - 1 splits between adjacent
// codes. A subtree over leaves [l, r] hangs below the split r (it is the left
// child) when delta(r, r+1) > delta(l-1, l), else below the split l - 1 (the
// right child); deltas past either end count as -1. Each leaf climbs: at its
// parent split it leaves its far bound in a slot with an atomic exchange; the
// first of the two children to arrive stops there, the second reads its
// sibling's bound and forms the node [L, R] with split p. This builds the
// unique binary radix tree over distinct sorted keys, which is the tree the
// reference's per-node searches produce for every node i >= 1; the node's
// index is R when it is a left child and L when it is a right child (the
// numbering of those searches), so it writes prefixN = delta(L, R),
// leftChild = p, the two leaf flags, parent[] of its internal children and
// their edge counts prefixN(child)/3 - prefixN(node)/3.
//
// Node 0 is the reference's special root: it spans keys [0, n-1], not
// [0, n]. When the true root splits at p < n-1 it makes the same split (only
// hasLeafRight can differ); when p = n-1 ("short root") node 0 repeats node
// n-1 = keys [0, n-1]. The thread that forms the true root writes node 0 that
// way; parent[] then equals the reference's (whose short-root writes node n-1
// wins, and whose unwritten entries are the zeros the true root writes).
// --------------------------------------------------------------------------
struct BuOut {
  uint8_t* prefix_n;
  uint8_t* hll;
  uint8_t* hlr;
  int* left_child;
  int* parent;
  int* ec;
};

struct SmemCodes {
  const uint32_t* s;  // codes[base, base + size)
  int base;
  __device__ __forceinline__ uint32_t operator[](int j) const { return s[j - base]; }
};

// delta between leaves k and k + 1, -1 past either end (N leaves)
template <class Codes>
__device__ __forceinline__ int bu_delta(const Codes& c, int k, int N) {
  return (k < 0 || k > N - 2) ? -1 : delta_u8(c[k], c[k + 1]);
}

// Node 0 from the true root (split p over leaves [0, N-1]).
template <class Codes>
__device__ __forceinline__ void bu_root(const Codes& c, int N, int p, const BuOut& o) {
  const int n = N - 1;
  o.parent[0] = 0;
  o.ec[0] = 0;
  const uint32_t c0 = c[0];
  if (n == 1) {  // one node over keys {0, 0}: clz(0) taken as 32
    o.prefix_n[0] = (uint8_t)delta_u8(c0, c0);
    o.left_child[0] = 0;
    o.hll[0] = 1;
    o.hlr[0] = 0;
    return;
  }
  const int pn0 = delta_u8(c0, c[n - 1]);
  o.prefix_n[0] = (uint8_t)pn0;
  if (p < n - 1) {
    o.left_child[0] = p;
    o.hll[0] = p == 0;
    o.hlr[0] = p + 1 == n - 1;
    if (p != 0) {
      o.parent[p] = 0;
      o.ec[p] = delta_u8(c0, c[p]) / 3 - pn0 / 3;
    }
    o.parent[p + 1] = 0;  // keys [p+1, n]: at least two
    o.ec[p + 1] = delta_u8(c[p + 1], c[n]) / 3 - pn0 / 3;
  } else {
    // short root: node n-1 (keys [0, n-1]) was formed before its parent; its
    // former fenced after writing leftChild[n-1], so fence and read it past L1
    __threadfence();
    const int g = (int)__ldcg(reinterpret_cast<const unsigned int*>(o.left_child + n - 1));
    o.left_child[0] = g;
    o.hll[0] = g == 0;
    o.hlr[0] = g + 1 == n - 1;
    o.parent[n - 1] = 0;
    o.ec[n - 1] = 0;  // prefixN[n-1] == prefixN[0]
  }
}

// Form node [L, R] with split p; true when it was the root (climb over).
template <class Codes>
__device__ __forceinline__ bool bu_form(const Codes& c, int N, int L, int R, int p,
                                        const BuOut& o) {
  if (L == 0 && R == N - 1) {
    bu_root(c, N, p, o);
    return true;
  }
  const int kidx = bu_delta(c, R, N) > bu_delta(c, L - 1, N) ? R : L;
  const uint32_t cL = c[L], cR = c[R];
  const int pn = delta_u8(cL, cR);
  o.prefix_n[kidx] = (uint8_t)pn;
  o.left_child[kidx] = p;
  o.hll[kidx] = L == p;
  o.hlr[kidx] = R == p + 1;
  if (L != p) {
    o.parent[p] = kidx;
    o.ec[p] = delta_u8(cL, c[p]) / 3 - pn / 3;
  }
  if (R != p + 1) {
    o.parent[p + 1] = kidx;
    o.ec[p + 1] = delta_u8(c[p + 1], cR) / 3 - pn / 3;
  }
  if (L == 0 && R == N - 2) __threadfence();  // node n-1 of a short root: see bu_root
  return false;
}

// Climb with global slots from an arrival at split p carrying bound `mine`
// (the child's range is [mine, p] or [p + 1, mine]).
template <class Codes>
__device__ __forceinline__ void bu_climb_global(const Codes& c, int N, int p, uint32_t mine,
                                                const BuOut& o, uint32_t* slot) {
  for (int guard = 0; guard < 64; ++guard) {
    const uint32_t prev = atomicExch(&slot[p], mine + 1u);
    if (prev == 0) return;
    const bool was_left = (int)mine <= p;
    const int L = was_left ? (int)mine : (int)prev - 1;
    const int R = was_left ? (int)prev - 1 : (int)mine;
    if (L < 0 || R >= N || L > p || R <= p) return;  // never for a zeroed slot array
    if (bu_form(c, N, L, R, p, o)) return;
    const bool left = bu_delta(c, R, N) > bu_delta(c, L - 1, N);
    p = left ? R : L - 1;
    mine = left ? (uint32_t)L : (uint32_t)R;
  }
}

}  // namespace octgb
