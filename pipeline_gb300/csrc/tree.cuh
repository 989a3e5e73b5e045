// Karras radix-tree node construction shared by the single-cloud and the
// batched builds.
#pragma once

#include "kernels.cuh"

namespace octgb {

// Delta-based tree (csrc/tree_tiled.cu): tiles of 4,096 positions, whose
// smallest deltas are scanned 512 at a time.
constexpr int kTtTile = 4096;
constexpr int kTtMinBlock = 512;
// D of a position past the last one (and of malformed pairs): never below a
// query value, which is at most 30 for codes below 2^31.
constexpr uint32_t kTtAbsent = 31;
__device__ __forceinline__ uint32_t tt_delta(uint32_t a, uint32_t b) {
  return min((uint32_t)delta_u8(a, b), kTtAbsent);
}

// Byte-wise minimum on the containing 32-bit word.
__device__ __forceinline__ void atomic_min_u8(uint8_t* addr, uint32_t v) {
  uint32_t* w = reinterpret_cast<uint32_t*>(reinterpret_cast<uintptr_t>(addr) & ~uintptr_t(3));
  const int sh = (int)(reinterpret_cast<uintptr_t>(addr) & 3) * 8;
  uint32_t old = *reinterpret_cast<volatile uint32_t*>(w);
  for (int it = 0; it < 4096; ++it) {  // retries only while other CTAs update the word
    if (((old >> sh) & 0xffu) <= v) return;
    const uint32_t assumed = old;
    old = atomicCAS(w, assumed, (assumed & ~(0xffu << sh)) | (v << sh));
    if (old == assumed) return;
  }
}

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

}  // namespace octgb
