// Octree stage (7-8) device functions shared by the single-cloud and the
// batched builds: sequence tags, per-node write emission, per-slot finalize.
#pragma once

#include "kernels.cuh"

namespace octgb {

constexpr uint32_t kLinkTag = 0x80000000u;

struct Sizes {
  int n_brt, n_oct;
  bool fits;
};

__device__ __forceinline__ Sizes read_sizes(const OctArgs& a) {
  Sizes z;
  z.n_brt = a.d_unique ? max(*a.d_unique - 1, 0) : a.n_brt_host;
  if (a.d_max_slot)
    z.n_oct = z.n_brt >= 1 ? *a.d_max_slot + 1 : 0;
  else
    z.n_oct = a.n_oct_host;
  z.fits = z.n_oct <= a.cap;
  return z;
}

__device__ __forceinline__ void put_child(const OctTags& t, int slot, int which, uint32_t tag,
                                          int n_oct, uint32_t* status) {
  if ((unsigned)slot >= (unsigned)n_oct) {
    raise_status(status, kStatusCapacity);
    return;
  }
  atomicMax(&t.child[(size_t)slot * 8 + which], tag);
}

// Every write radix node i makes (MakeOctNodes for i >= 1 when mode has
// kOctMake, LinkLeafNodes when it has kOctLink), as tags.
//
// Loads are grouped by dependency so each round is issued at once: the node's
// own entries; then its parent's count and parent link and the codes of its
// leaf children; then the rest of the walk up to the first radix node with
// octree nodes (usually none); then that node's octree offset. At most one
// walk applies: MakeOctNodes walks from parent[i] when i has octree nodes,
// LinkLeafNodes walks from i, i.e. from parent[i] when i has none.
__device__ __forceinline__ void emit_node(int mode, int i, const OctArgs& a, const OctTags& t,
                                          const Sizes& z, uint32_t* status) {
  const int pn = a.prefix_n[i];
  const int k = a.counts[i];
  const int par = a.parent[i];
  const bool make = (mode & kOctMake) && i >= 1 && k > 0;
  const bool ll = (mode & kOctLink) && a.hll[i];
  const bool lr = (mode & kOctLink) && a.hlr[i];
  const bool link = ll || lr;
  int base = 0, lc = 0;
  uint32_t code = 0;
  if (make) {
    base = a.offsets[i];
    code = a.codes[i];
  }
  if (link) lc = a.left_child[i];
  const int L = pn / 3;
  // walk start: the parent (MakeOctNodes; LinkLeafNodes of a node without
  // octree nodes other than 0) or i itself (LinkLeafNodes otherwise)
  const bool walk_link = link && k == 0 && i != 0;
  const bool walk = make || walk_link;
  int wc = 0, wp = 0;
  uint32_t cl = 0, cr = 0;
  const bool lc_ok = (unsigned)lc < (unsigned)z.n_brt;  // leaf index lc + 1 <= n_brt
  const bool par_ok = (unsigned)par < (unsigned)z.n_brt;
  if (walk && par_ok) {
    wc = a.counts[par];
    wp = a.parent[par];
  }
  if (link && lc_ok) {
    if (ll) cl = a.codes[lc];
    if (lr) cr = a.codes[lc + 1];
  }

  if (make) {
    // include/shared/oct.h:24-90
    for (int j = 0; j < k - 1; ++j) {
      const int level = L - j;
      const uint32_t pre = code >> (30 - 3 * level);
      const int which = (int)(pre & 7u);
      const int up = base + j + 1;
      put_child(t, up, which, (((uint32_t)i << 4) | (uint32_t)j) + 1u, z.n_oct, status);
      if ((unsigned)up < (unsigned)z.n_oct) atomicOr(&t.mask[up], 1u << which);
      if ((unsigned)(base + j) < (unsigned)z.n_oct) atomicMax(&t.owner[base + j], (uint32_t)i);
    }
    int rp = par;
    bool bad = !par_ok;
    if (!bad && wc == 0) {
      int counter = 0;
      rp = wp;
      bad = (unsigned)rp >= (unsigned)z.n_brt;
      if (!(++counter > 30))
        while (!bad && a.counts[rp] == 0) {
          rp = a.parent[rp];
          bad = (unsigned)rp >= (unsigned)z.n_brt;
          if (++counter > 30) break;
        }
    }
    if (bad) {  // malformed parent[]: never read out of bounds
      raise_status(status, kStatusWalkLimit);
      rp = 0;
    }
    const int top = L - k + 1;
    const int which = (int)((code >> (30 - 3 * top)) & 7u);
    const int oct_parent = a.offsets[rp];
    put_child(t, oct_parent, which, (((uint32_t)i << 4) | (uint32_t)(k - 1)) + 1u, z.n_oct,
              status);
    if ((unsigned)oct_parent < (unsigned)z.n_oct) atomicOr(&t.mask[oct_parent], 1u << which);
    const int slot = base + k - 1;
    if ((unsigned)slot < (unsigned)z.n_oct) atomicMax(&t.owner[slot], (uint32_t)i);
    else raise_status(status, kStatusCapacity);
  }
  if (link) {
    // include/shared/oct.h:92-134, walk bounded at radix node 0.
    int rn = i;
    if (walk_link) {
      int steps = 0;
      if (!par_ok) {
        raise_status(status, kStatusWalkLimit);
      } else {
        rn = par;
        ++steps;
        int cnt = wc, up = wp;
        while (cnt == 0 && rn != 0) {
          if ((unsigned)up >= (unsigned)z.n_brt || ++steps > 64) {
            raise_status(status, kStatusWalkLimit);
            break;
          }
          rn = up;
          cnt = a.counts[rn];
          up = a.parent[rn];
        }
      }
    }
    // rn == i with octree nodes: its offset is already in base (a load here
    // would wait behind the MakeOctNodes atomics, which the compiler may not
    // move it above).
    const int dst = (make && rn == i) ? base : a.offsets[rn];
    const uint32_t sh = (uint32_t)(30 - 3 * (L + 1)) & 31u;
    if (!lc_ok) {
      raise_status(status, kStatusWalkLimit);
      return;
    }
    if (ll) put_child(t, dst, (int)((cl >> sh) & 7u), kLinkTag | ((uint32_t)i << 1), z.n_oct, status);
    if (lr)
      put_child(t, dst, (int)((cr >> sh) & 7u), kLinkTag | ((uint32_t)i << 1) | 1u, z.n_oct,
                status);
  }
}

// range / 2^k as the reference computes it (float division by (float)(1 << k)).
// For k in [0, 30] the divisor is the exact power of two, and the correctly
// rounded quotient equals the correctly rounded product range * 2^-k.
__device__ __forceinline__ float cell_size(float range, int k) {
  if (k >= 0 && k <= 30) return __fmul_rn(range, __int_as_float((127 - k) << 23));
  return __fdiv_rn(range, (float)(1 << k));
}

// One thread per slot computes the node; the block stages its 256 nodes
// (15 KB) in shared memory and writes them as consecutive 32-bit words, so
// every warp store is one contiguous 128-byte line.
constexpr int kFinThreads = 256;
constexpr int kNodeWords = 15;

// The 15 words of slot p (children, corner, cell_size, masks) into w.
__device__ __forceinline__ void finalize_slot(bool fresh, int p, const OctArgs& a,
                                              const OctTags& t, int root_level, int* w) {
  const uint4* c4 = reinterpret_cast<const uint4*>(t.child);
  const uint4 ta = c4[2 * p], tb = c4[2 * p + 1];
  const uint32_t tags[8] = {ta.x, ta.y, ta.z, ta.w, tb.x, tb.y, tb.z, tb.w};
  const oct_node* nd = a.nodes + p;
  const uint32_t m = t.mask[p];
  const uint32_t own = t.owner[p];
  // Every table read below depends only on the tags: issue them all at once.
  int base[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const uint32_t g = tags[c];
    const int* src = (g & kLinkTag) ? a.left_child + ((g & ~kLinkTag) >> 1)
                                    : a.offsets + ((g - 1u) >> 4);
    base[c] = 0;
    if (g != 0) base[c] = __ldg(src);
  }
  int own_off = 0, own_pn = 0;
  uint32_t own_code = 0;
  if (own != 0) {
    own_off = __ldg(a.offsets + own);
    own_pn = __ldg(a.prefix_n + own);
    own_code = __ldg(a.codes + own);
  }
  uint32_t link_bits = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const uint32_t g = tags[c];
    int v;
    if (g == 0) {
      v = fresh ? 0 : nd->children[c];
    } else if (g & kLinkTag) {
      v = base[c] + (int)(g & 1u);
      link_bits |= 1u << c;
    } else {
      v = base[c] + (int)((g - 1u) & 15u);
    }
    w[c] = v;
  }
  float4 corner;
  float cell;
  if (own != 0) {
    const int j = p - own_off;
    const int level = own_pn / 3 - j;
    const int sh = 30 - 3 * level;
    corner = decode_corner((own_code >> sh) << sh, a.min_coord, a.range);
    cell = cell_size(a.range, level - root_level);
  } else if (fresh && p == 0) {
    const int sh = 30 - 3 * root_level;
    corner = decode_corner((a.codes[0] >> sh) << sh, a.min_coord, a.range);
    cell = a.range;
  } else if (fresh) {
    corner = make_float4(0.f, 0.f, 0.f, 0.f);
    cell = 0.f;
  } else {
    corner = make_float4(nd->corner.x, nd->corner.y, nd->corner.z, nd->corner.w);
    cell = nd->cell_size;
  }
  w[8] = __float_as_int(corner.x);
  w[9] = __float_as_int(corner.y);
  w[10] = __float_as_int(corner.z);
  w[11] = __float_as_int(corner.w);
  w[12] = __float_as_int(cell);
  if (fresh) {
    w[13] = (int)m;
    w[14] = 0;
  } else {
    w[13] = nd->child_node_mask | (int)m;
    w[14] = nd->child_leaf_mask & ~(int)link_bits;
  }
}

}  // namespace octgb
