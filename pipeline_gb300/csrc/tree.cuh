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
__device__ __forceinline__ void radix_node(int i, int n, const uint32_t* __restrict__ codes,
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
      const long long e = (long long)i + (long long)lmax * d;
      if (e < 0 || e > n || delta_u8(ci, codes[e]) <= dmin) break;
      lmax *= 2;
    }
    const int lcut = (d == -1) ? i : n - i;
    for (unsigned div = 2, t = (unsigned)lmax / 2; t >= 1; div *= 2, t = (unsigned)lmax / div)
      if (l + (int)t <= lcut && delta_u8(ci, codes[i + (l + (int)t) * d]) > dmin) l += (int)t;
  }
  const int j = i + l * d;
  const int dnode = delta_u8(ci, codes[j]);
  prefix_n[i] = (uint8_t)dnode;
  int s = 0;
  if (l > 0) {
    const unsigned maxdiv = 1u << log2_ceil_u32((uint32_t)l);
    const int scut = (d == -1) ? i - 1 : n - i - 1;
    for (unsigned div = 2, t = ((unsigned)l + 1) / 2; div <= maxdiv;
         div <<= 1, t = ((unsigned)l + div - 1) / div)
      if (s + (int)t <= scut && delta_u8(ci, codes[i + (s + (int)t) * d]) > dnode) s += (int)t;
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
