// Stages 7-8 of whole builds: octree nodes and leaf links in shared memory.
//
// Replaces k_MakeOctNodes / k_LinkLeafNodes (reference
// include/kernels/07_octree.hpp:5-25, include/shared/oct.h:9-134) and the
// caller's root set-up (apps/cpu_demo/main.cpp:125-132) for radix trees this
// library built itself (whole and learned builds); the stage entry points,
// which accept any arrays, keep the tag form of octree.cu.
//
// The result is the one of a sequential run in ascending radix-node order
// (LinkLeaf's left write before its right one, every LinkLeaf write after
// every MakeOctNodes write): per OctNode child, the write with the largest
// sequence tag (octree.cuh) wins; corner and cell_size come from the largest
// radix node whose slot range covers the slot; child_node_mask is the OR of
// every SetChild bit; child_leaf_mask stays 0.
//
// Radix node i with k_i = edge_count[i] > 0 writes the slots
// [P_i, P_i + k_i - 1], P_i = prefix_sum[i] (inclusive, so the ranges of
// consecutive nodes can overlap): their corners, and a child of each slot
// but the first (the chain); its top slot becomes a child of the first slot
// of its nearest ancestor r with k_r > 0 (the group root; 0 for the root's
// group), and its leaves become children of the first slot of i itself (or
// of its group root when k_i = 0). P is strictly increasing over the nodes
// with k > 0, so every write but the group-root ones lands near P_i.
//
// oct_tile_kernel: one CTA per tile of kOtTile consecutive radix nodes (one
// thread each), which owns the slots (P_{i0-1}, P_{i1-1}] (the last tile: up
// to M - 1). The tile's node fields are staged in shared memory, so the walks
// to group roots (usually one or two steps up, mostly inside the tile) read
// shared memory. Its slots are built there too, in chunks of kOtChunk slots:
// every write that lands in the chunk, from the tile's nodes and from the few
// nodes before it whose ranges reach into it, is merged by shared-memory
// atomicMax on 32-bit sequence tags; the chunk's OctNodes are then derived
// from the winning tags (a tag names its writer and step, whose value is the
// writer's offset plus the step, or its left child plus the side) and written
// once, coalesced. A group-root write whose slot belongs to another tile
// (about 1% of them) instead flags that slot, and the root's slot 0 takes its
// writes in a small global block (64-bit words: tag << 32 | value).
//
// oct_fixup_kernel: rebuilds every flagged slot, and slot 0, from scratch
// after all tiles are done, one warp per slot: the ranges covering it (a
// backward scan of the prefix sums), then the group-root writes by walking
// down from the slot's radix node through its descendants with k = 0 (at
// most two levels for unique codes: prefixes within one octal digit), a level
// at a time across the lanes.
#include "octree.cuh"

namespace octgb {

constexpr int kOtThreads = 512;  // radix nodes per tile, one per thread
constexpr int kOtTile = kOtThreads;
constexpr int kOtChunk = 512;    // slots per shared-memory pass
constexpr int kOtHalo = 64;      // halo nodes staged in shared memory

size_t oct_fix_zero_bytes(int cap) {
  const size_t words = (size_t)(cap > 0 ? cap : 1) / 32 + 1;
  return align_up(128 + 4 * words, 256);
}

size_t oct_fix_list_bytes(int cap) { return align_up(4 * (size_t)(cap > 0 ? cap : 1), 256); }

OctFix oct_fix_carve(void* zeroed, void* list, int cap) {
  char* z = static_cast<char*>(zeroed);
  OctFix f;
  f.root_child = reinterpret_cast<unsigned long long*>(z);
  f.root_mask = reinterpret_cast<uint32_t*>(z + 64);
  f.count = reinterpret_cast<uint32_t*>(z + 68);
  f.flags = reinterpret_cast<uint32_t*>(z + 128);
  f.list = static_cast<int*>(list);
  f.cap = cap;
  return f;
}

namespace {

struct OtSmem {
  union {
    struct {
      uint32_t child[8 * kOtChunk];  // tag of child c of chunk slot x at [c * kOtChunk + x]
      uint32_t owner[kOtChunk];      // largest radix node covering the slot (0 = none)
      uint32_t mask[kOtChunk];       // OR of SetChild bits
    } t;
    int stage[kOtChunk * kNodeWords];  // the chunk's OctNodes, once the tags are read
  } u;
  // the tile's radix nodes [i0, i1) and codes [i0, i1]
  int cnt[kOtTile];
  int par[kOtTile];
  int off[kOtTile];
  int lc[kOtTile];
  uint32_t code[kOtTile + 1];
  uint8_t pn[kOtTile];
  // halo nodes [hs, i0) when there are at most kOtHalo
  int h_cnt[kOtHalo];
  int h_off[kOtHalo];
  uint32_t h_code[kOtHalo];
  uint8_t h_pn[kOtHalo];
  int hs;
};

__device__ __forceinline__ unsigned long long cw(uint32_t tag, uint32_t value) {
  return ((unsigned long long)tag << 32) | value;
}

__device__ __forceinline__ int octant(uint32_t code, int level) {
  return (int)((code >> (uint32_t)(30 - 3 * level)) & 7u);
}

__device__ __forceinline__ uint32_t make_tag(int i, int j) {
  return (((uint32_t)i << 4) | (uint32_t)j) + 1u;
}

// Radix-node fields, from shared memory for the tile's nodes (and the staged
// halo), else from global memory.
struct Tile {
  const OtSmem& sm;
  const OctArgs& a;
  int i0, i1, hs;
  bool halo;  // halo staged
  __device__ __forceinline__ bool in(int x) const {
    return (unsigned)(x - i0) < (unsigned)(i1 - i0);
  }
  __device__ __forceinline__ bool in_halo(int x) const {
    return halo && (unsigned)(x - hs) < (unsigned)(i0 - hs);
  }
  __device__ __forceinline__ int cnt(int x) const {
    return in(x) ? sm.cnt[x - i0] : in_halo(x) ? sm.h_cnt[x - hs] : a.counts[x];
  }
  __device__ __forceinline__ int par(int x) const { return in(x) ? sm.par[x - i0] : a.parent[x]; }
  __device__ __forceinline__ int off(int x) const {
    return in(x) ? sm.off[x - i0] : in_halo(x) ? sm.h_off[x - hs] : a.offsets[x];
  }
  __device__ __forceinline__ int pn(int x) const {
    return in(x) ? sm.pn[x - i0] : in_halo(x) ? sm.h_pn[x - hs] : a.prefix_n[x];
  }
  __device__ __forceinline__ uint32_t code(int x) const {
    return (unsigned)(x - i0) <= (unsigned)(i1 - i0) ? sm.code[x - i0]
           : in_halo(x)                             ? sm.h_code[x - hs]
                                                    : a.codes[x];
  }
};

// Chain / owner writes of radix node i (slot range [P, P + k - 1], level L at
// slot P) that land in the chunk [c0, c1).
__device__ __forceinline__ void chain_writes(OtSmem& sm, int i, int P, int k, int L, uint32_t code,
                                             int c0, int c1) {
  const int lo = max(P, c0), hi = min(P + k - 1, c1 - 1);
  for (int s = lo; s <= hi; ++s) {
    atomicMax(&sm.u.t.owner[s - c0], (uint32_t)i);
    if (s > P) {  // SetChild(slot s, octant of level L - j, value s - 1), j = s - P - 1
      const int j = s - P - 1;
      const int c = octant(code, L - j);
      atomicMax(&sm.u.t.child[c * kOtChunk + (s - c0)], make_tag(i, j));
      atomicOr(&sm.u.t.mask[s - c0], 1u << c);
    }
  }
}

// Group root for MakeOctNodes' walk (include/shared/oct.h:52-63): from the
// parent, up while the count is 0, at most 31 steps; node 0 when the walk
// leaves the array.
__device__ __forceinline__ int make_walk(const Tile& t, int par, int n_brt, uint32_t* status) {
  if ((unsigned)par >= (unsigned)n_brt) {
    raise_status(status, kStatusWalkLimit);
    return 0;
  }
  int rp = par;
  int counter = 0;
  while (t.cnt(rp) == 0) {
    const int up = t.par(rp);
    if ((unsigned)up >= (unsigned)n_brt) {
      raise_status(status, kStatusWalkLimit);
      return 0;
    }
    rp = up;
    if (++counter > 30) break;
  }
  return rp;
}

// Group root for LinkLeafNodes' walk (oct.h:111-113), bounded at node 0.
__device__ __forceinline__ int link_walk(const Tile& t, int par, int n_brt, uint32_t* status) {
  if ((unsigned)par >= (unsigned)n_brt) {
    raise_status(status, kStatusWalkLimit);
    return 0;
  }
  int rn = par;
  int steps = 1;
  while (rn != 0 && t.cnt(rn) == 0) {
    const int up = t.par(rn);
    if ((unsigned)up >= (unsigned)n_brt || ++steps > 64) {
      raise_status(status, kStatusWalkLimit);
      return 0;
    }
    rn = up;
  }
  return rn;
}

// A write into slot `dest` outside the tile's slots: slot 0 takes it in the
// global root block, any other slot is flagged for the fix-up (its radix node
// `root` listed once). Warp-aggregated list appends; every lane calls this.
__device__ __forceinline__ void remote_push(const OctFix& f, int dest, int root, int c,
                                            uint32_t tag, uint32_t val, bool make, bool active,
                                            uint32_t* status) {
  if (!__any_sync(0xffffffffu, active)) return;  // the common case: all local
  bool append = false;
  if (active) {
    if (dest == 0) {
      atomicMax(&f.root_child[c], cw(tag, val));
      if (make) atomicOr(f.root_mask, 1u << c);
    } else if ((unsigned)dest < (unsigned)f.cap) {
      const uint32_t bit = 1u << (dest & 31);
      append = !(atomicOr(&f.flags[dest >> 5], bit) & bit);
    } else {
      raise_status(status, kStatusCapacity);
    }
  }
  const uint32_t m = __ballot_sync(0xffffffffu, append);
  if (m) {
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(f.count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (append) f.list[base + __popc(m & lanemask_lt())] = root;
  }
}

}  // namespace

__global__ void __launch_bounds__(kOtThreads, 3)
    oct_tile_kernel(OctArgs a, OctFix f, uint32_t* __restrict__ status, int tile_nodes,
                    int chunk_slots) {
  extern __shared__ __align__(16) unsigned char ot_smem_raw[];
  OtSmem& sm = *reinterpret_cast<OtSmem*>(ot_smem_raw);
  const Sizes z = read_sizes(a);
  const int B = z.n_brt, M = z.n_oct;
  if (!z.fits) {
    if (blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, kStatusCapacity);
    return;
  }
  const int i0 = blockIdx.x * tile_nodes;
  if (B < 1 || i0 >= B) return;
  const int i1 = min(i0 + tile_nodes, B);
  const int tn = i1 - i0;
  const int tid = threadIdx.x;
  const int w0 = i0 == 0 ? 1 : a.offsets[i0 - 1] + 1;
  const int w1 = i1 == B ? M : a.offsets[i1 - 1] + 1;
  const int root_level = a.prefix_n[0] / 3;

  // This thread's radix node, staged for the others.
  const bool home = tid < tn;
  const int i = i0 + tid;
  int k = 0, L = 0, P = 0, par = 0, lc = 0;
  uint32_t code = 0;
  bool hl = false, hr = false;
  if (home) {
    k = a.counts[i];
    par = a.parent[i];
    P = a.offsets[i];
    const int pnv = a.prefix_n[i];
    L = pnv / 3;
    code = a.codes[i];
    hl = a.hll[i];
    hr = a.hlr[i];
    if (hl || hr) lc = a.left_child[i];
    sm.cnt[tid] = k;
    sm.par[tid] = par;
    sm.off[tid] = P;
    sm.pn[tid] = (uint8_t)pnv;
    sm.code[tid] = code;
    sm.lc[tid] = lc;
  }
  if (tid == 0) sm.code[tn] = a.codes[i1];  // U = B + 1 codes
  // Halo: the nodes before the tile whose ranges can reach its first slot,
  // i.e. with P >= w0 - 9 (a range spans at most 10 slots): a backward scan
  // of the non-decreasing prefix sums, 32 nodes a round.
  if (tid < 32) {
    const int key = w0 - 9;
    int hs = i0;
    for (int base = i0 - 1; base >= 0; base -= 32) {
      const int x = base - tid;
      const uint32_t m = __ballot_sync(0xffffffffu, x >= 0 && a.offsets[x] >= key);
      if (m != 0xffffffffu) {
        hs = base - (__ffs(~m) - 1) + 1;  // the lanes before the first miss are halo nodes
        break;
      }
      hs = base - 31;
    }
    if (tid == 0) sm.hs = hs;
    const int H = i0 - hs;
    if (H <= kOtHalo) {
      for (int x = tid; x < H; x += 32) {
        sm.h_cnt[x] = a.counts[hs + x];
        sm.h_off[x] = a.offsets[hs + x];
        sm.h_pn[x] = a.prefix_n[hs + x];
        sm.h_code[x] = a.codes[hs + x];
      }
    }
  }
  for (int x = tid; x < min(chunk_slots, max(w1 - w0, 0)); x += kOtThreads) {
#pragma unroll
    for (int c = 0; c < 8; ++c) sm.u.t.child[c * kOtChunk + x] = 0u;
    sm.u.t.owner[x] = 0u;
    sm.u.t.mask[x] = 0u;
  }
  __syncthreads();
  const int hs = sm.hs;
  const Tile t{sm, a, i0, i1, hs, i0 - hs <= kOtHalo};

  for (int c0 = w0; c0 < w1; c0 += chunk_slots) {
    const int c1 = min(c0 + chunk_slots, w1);
    const int cn = c1 - c0;
    if (c0 != w0) {  // later chunks (windows longer than a chunk): clear again
      for (int x = tid; x < cn; x += kOtThreads) {
#pragma unroll
        for (int c = 0; c < 8; ++c) sm.u.t.child[c * kOtChunk + x] = 0u;
        sm.u.t.owner[x] = 0u;
        sm.u.t.mask[x] = 0u;
      }
      __syncthreads();
    }
    // halo nodes: their ranges only
    for (int h = hs + tid; h < i0; h += kOtThreads) {
      const int kh = t.cnt(h);
      if (h >= 1 && kh > 0) {
        const int Ph = t.off(h);
        if (Ph + kh - 1 >= c0) chain_writes(sm, h, Ph, kh, t.pn(h) / 3, t.code(h), c0, c1);
      }
    }
    // this thread's node: its range, its top slot's link, its leaves
    int t_dest = -1, t_root = 0, t_c = 0;
    int l_dest = -1, l_root = 0, l_c = -1, r_c = -1;
    if (home) {
      if (i >= 1 && k > 0) {
        chain_writes(sm, i, P, k, L, code, c0, c1);
        const int rp = make_walk(t, par, B, status);
        if (rp != 0 && t.cnt(rp) == 0) raise_status(status, kStatusWalkLimit);  // not a group root
        t_root = rp;
        t_dest = t.off(rp);
        t_c = octant(code, L - k + 1);
        if (t_dest >= c0 && t_dest < c1) {
          atomicMax(&sm.u.t.child[t_c * kOtChunk + (t_dest - c0)], make_tag(i, k - 1));
          atomicOr(&sm.u.t.mask[t_dest - c0], 1u << t_c);
        }
      }
      if (hl || hr) {
        if ((unsigned)lc >= (unsigned)B) {  // leaf index lc + 1 <= B
          raise_status(status, kStatusWalkLimit);
        } else {
          const bool own = k > 0 || i == 0;
          l_root = own ? i : link_walk(t, par, B, status);
          l_dest = own ? P : t.off(l_root);
          const uint32_t sh = (uint32_t)(30 - 3 * (L + 1)) & 31u;
          if (hl) l_c = (int)((t.code(lc) >> sh) & 7u);
          if (hr) r_c = (int)((t.code(lc + 1) >> sh) & 7u);
          if (l_dest >= c0 && l_dest < c1) {
            if (hl)
              atomicMax(&sm.u.t.child[l_c * kOtChunk + (l_dest - c0)],
                        kLinkTag | ((uint32_t)i << 1));
            if (hr)
              atomicMax(&sm.u.t.child[r_c * kOtChunk + (l_dest - c0)],
                        kLinkTag | ((uint32_t)i << 1) | 1u);
          }
        }
      }
    }
    if (c0 == w0) {  // writes into other tiles' slots, once
      remote_push(f, t_dest, t_root, t_c, make_tag(i, k - 1), (uint32_t)(P + k - 1), true,
                  t_dest >= 0 && (t_dest < w0 || t_dest >= w1), status);
      const bool lrem = l_dest >= 0 && (l_dest < w0 || l_dest >= w1);
      remote_push(f, l_dest, l_root, l_c, kLinkTag | ((uint32_t)i << 1), (uint32_t)lc, false,
                  lrem && l_c >= 0, status);
      remote_push(f, l_dest, l_root, r_c, kLinkTag | ((uint32_t)i << 1) | 1u, (uint32_t)(lc + 1),
                  false, lrem && r_c >= 0, status);
    }
    __syncthreads();
    // the chunk's OctNodes: one slot a thread, in registers first (the stage
    // reuses the tags)
    int words[kNodeWords];
    const int x = tid;
    if (x < cn) {
      const int p = c0 + x;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const uint32_t g = sm.u.t.child[c * kOtChunk + x];
        int v = 0;
        if (g & kLinkTag) {
          const int w = (int)((g & ~kLinkTag) >> 1);
          v = (t.in(w) ? sm.lc[w - i0] : a.left_child[w]) + (int)(g & 1u);
        } else if (g != 0) {
          v = t.off((int)((g - 1u) >> 4)) + (int)((g - 1u) & 15u);
        }
        words[c] = v;
      }
      const int own = (int)sm.u.t.owner[x];
      float4 corner = make_float4(0.f, 0.f, 0.f, 0.f);
      float cell = 0.f;
      if (own != 0) {
        const int level = t.pn(own) / 3 - (p - t.off(own));
        const int sh = 30 - 3 * level;
        corner = decode_corner((t.code(own) >> sh) << sh, a.min_coord, a.range);
        cell = cell_size(a.range, level - root_level);
      }
      words[8] = __float_as_int(corner.x);
      words[9] = __float_as_int(corner.y);
      words[10] = __float_as_int(corner.z);
      words[11] = __float_as_int(corner.w);
      words[12] = __float_as_int(cell);
      words[13] = (int)sm.u.t.mask[x];
      words[14] = 0;
    }
    __syncthreads();
    if (x < cn) {
#pragma unroll
      for (int w = 0; w < kNodeWords; ++w) sm.u.stage[x * kNodeWords + w] = words[w];
    }
    __syncthreads();
    // coalesced copy-out: 16-byte vectors when the destination is aligned
    int* dst = reinterpret_cast<int*>(a.nodes) + (size_t)c0 * kNodeWords;
    const int nw = cn * kNodeWords;
    if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
      const int quads = nw >> 2;
      const uint4* s4 = reinterpret_cast<const uint4*>(sm.u.stage);
      uint4* d4 = reinterpret_cast<uint4*>(dst);
      for (int q = tid; q < quads; q += kOtThreads) d4[q] = s4[q];
      for (int q = (quads << 2) + tid; q < nw; q += kOtThreads) dst[q] = sm.u.stage[q];
    } else {
      for (int q = tid; q < nw; q += kOtThreads) dst[q] = sm.u.stage[q];
    }
    __syncthreads();
  }
}

namespace {

constexpr int kFxThreads = 256;
constexpr int kFxMembers = 16;  // group members per level (unique codes: at most 4)

// Writes one finished OctNode (fresh build: child_leaf_mask 0).
__device__ __forceinline__ void put_node(oct_node* nodes, int p, const unsigned long long* child,
                                         uint32_t mask, float4 corner, float cell) {
  int* w = reinterpret_cast<int*>(nodes + p);
#pragma unroll
  for (int c = 0; c < 8; ++c) w[c] = (int)(uint32_t)child[c];
  w[8] = __float_as_int(corner.x);
  w[9] = __float_as_int(corner.y);
  w[10] = __float_as_int(corner.z);
  w[11] = __float_as_int(corner.w);
  w[12] = __float_as_int(cell);
  w[13] = (int)mask;
  w[14] = 0;
}

// child[c] = max(child[c], w) for a run-time c, with the array kept in registers.
__device__ __forceinline__ void take(unsigned long long* child, int c, unsigned long long w) {
#pragma unroll
  for (int q = 0; q < 8; ++q)
    if (q == c && w > child[q]) child[q] = w;
}

}  // namespace

// Slot 0 from the root block; every flagged slot P_r from scratch, one warp
// per slot. Each lane keeps its own maxima of the child words it finds; the
// warp merges them at the end.
__global__ void __launch_bounds__(kFxThreads)
    oct_fixup_kernel(OctArgs a, OctFix f, uint32_t* __restrict__ status) {
  __shared__ int s_members[kFxThreads / 32][2][kFxMembers];
  const Sizes z = read_sizes(a);
  const int B = z.n_brt;
  if (!z.fits || B < 1) return;
  const int root_level = a.prefix_n[0] / 3;
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  if (gw == 0 && lane == 0) {  // the root: apps/cpu_demo/main.cpp:125-132 + writes into slot 0
    unsigned long long child[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) child[c] = f.root_child[c];
    const int sh = 30 - 3 * root_level;
    put_node(a.nodes, 0, child, *f.root_mask,
             decode_corner((a.codes[0] >> sh) << sh, a.min_coord, a.range), a.range);
  }
  const int n_list = (int)*f.count;
  for (int e = gw; e < n_list; e += nwarps) {
    const int r = f.list[e];
    if ((unsigned)r >= (unsigned)B) {
      if (lane == 0) raise_status(status, kStatusWalkLimit);
      continue;
    }
    const int p = a.offsets[r];
    unsigned long long child[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t mask = 0, own = 0;
    // ranges covering p: lane l looks at node base - l, nodes i <= r with
    // P_i >= p - 9 (a backward scan of the non-decreasing prefix sums)
    for (int base = r; base >= 0; base -= 32) {
      const int i = base - lane;
      int P = 0;
      const bool in = i >= 0 && (P = a.offsets[i]) >= p - 9;
      if (in && i >= 1) {
        const int k = a.counts[i];
        if (k > 0 && p <= P + k - 1) {
          own = max(own, (uint32_t)i);
          if (p > P) {
            const int j = p - P - 1;
            const int c = octant(a.codes[i], a.prefix_n[i] / 3 - j);
            take(child, c, cw(make_tag(i, j), (uint32_t)(p - 1)));
            mask |= 1u << c;
          }
        }
      }
      if (__ballot_sync(0xffffffffu, in) != 0xffffffffu) break;
    }
    // group-root writes: down from r through its descendants with k = 0, a
    // level at a time, one member a lane
    int nm = 1, buf = 0;
    if (lane == 0) s_members[wl][0][0] = r;
    __syncwarp();
    while (nm > 0) {
      int nw0 = -1, nw1 = -1;  // new members from this lane's two children
      if (lane < nm) {
        const int m = s_members[wl][buf][lane];
        const int lcm = a.left_child[m];
        const bool leaf0 = a.hll[m], leaf1 = a.hlr[m];
        const uint32_t sh = (uint32_t)(30 - 3 * (a.prefix_n[m] / 3 + 1)) & 31u;
#pragma unroll
        for (int side = 0; side < 2; ++side) {
          const int x = lcm + side;
          if (side == 0 ? leaf0 : leaf1) {
            if ((unsigned)x > (unsigned)B) {  // leaf index <= B
              raise_status(status, kStatusWalkLimit);
              continue;
            }
            take(child, (int)((a.codes[x] >> sh) & 7u),
                 cw(kLinkTag | ((uint32_t)m << 1) | (uint32_t)side, (uint32_t)x));
            continue;
          }
          if (x <= 0 || x >= B) {
            raise_status(status, kStatusWalkLimit);
            continue;
          }
          const int kx = a.counts[x];
          if (kx > 0) {
            const int c = octant(a.codes[x], a.prefix_n[x] / 3 - kx + 1);
            take(child, c, cw(make_tag(x, kx - 1), (uint32_t)(a.offsets[x] + kx - 1)));
            mask |= 1u << c;
          } else if (side == 0) {
            nw0 = x;
          } else {
            nw1 = x;
          }
        }
      }
      // gather the next level's members
      const uint32_t m0 = __ballot_sync(0xffffffffu, nw0 >= 0);
      const uint32_t m1 = __ballot_sync(0xffffffffu, nw1 >= 0);
      const int n0 = __popc(m0), n1 = __popc(m1);
      if (n0 + n1 > kFxMembers) {
        if (lane == 0) raise_status(status, kStatusWalkLimit);
        break;
      }
      const int nb = buf ^ 1;
      if (nw0 >= 0) s_members[wl][nb][__popc(m0 & lanemask_lt())] = nw0;
      if (nw1 >= 0) s_members[wl][nb][n0 + __popc(m1 & lanemask_lt())] = nw1;
      __syncwarp();
      nm = n0 + n1;
      buf = nb;
    }
    // merge the lanes
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      own = max(own, __shfl_xor_sync(0xffffffffu, own, o));
      mask |= __shfl_xor_sync(0xffffffffu, mask, o);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, child[c], o);
        if (v > child[c]) child[c] = v;
      }
    }
    if (lane == 0) {
      float4 corner = make_float4(0.f, 0.f, 0.f, 0.f);
      float cell = 0.f;
      if (own != 0) {
        const int level = a.prefix_n[own] / 3 - (p - a.offsets[own]);
        const int sh = 30 - 3 * level;
        corner = decode_corner((a.codes[own] >> sh) << sh, a.min_coord, a.range);
        cell = cell_size(a.range, level - root_level);
      }
      put_node(a.nodes, p, child, mask, corner, cell);
    }
    __syncwarp();
  }
}

namespace {
int g_tile_nodes = kOtTile;
int g_chunk_slots = kOtChunk;
}  // namespace

bool set_octree_tiling(int tile_nodes, int chunk_slots) {
  if (tile_nodes == 0 && chunk_slots == 0) {
    g_tile_nodes = kOtTile;
    g_chunk_slots = kOtChunk;
    return true;
  }
  if (tile_nodes < 1 || tile_nodes > kOtTile || chunk_slots < 1 || chunk_slots > kOtChunk)
    return false;
  g_tile_nodes = tile_nodes;
  g_chunk_slots = chunk_slots;
  return true;
}

cudaError_t launch_octree_tiled(const OctArgs& a, const OctFix& f, uint32_t* status,
                                cudaStream_t s, Recorder* rec) {
  const int nb = a.n_brt_host;
  const int tile_nodes = g_tile_nodes, chunk_slots = g_chunk_slots;
  int grid = (nb + tile_nodes - 1) / tile_nodes;
  if (grid < 1) grid = 1;
  const int smem = (int)sizeof(OtSmem);
  cudaError_t e = set_smem_limit(oct_tile_kernel, smem);
  if (e != cudaSuccess) return e;
  oct_tile_kernel<<<grid, kOtThreads, smem, s>>>(a, f, status, tile_nodes, chunk_slots);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  mark(rec, s);
  oct_fixup_kernel<<<device_sm_count() * 8, kFxThreads, 0, s>>>(a, f, status);
  e = cudaGetLastError();
  if (e == cudaSuccess) mark(rec, s);
  return e;
}

}  // namespace octgb
