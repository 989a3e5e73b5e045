// Stage 4 (and stage 5's edge counts) for strictly increasing codes below
// 2^31, from the deltas of adjacent codes.
//
// For such codes the radix tree of k_BuildRadixTree
// (kernels/04_radix_tree.cpp:39-121) is the Cartesian tree of the adjacent
// deltas D[q] = delta(codes[q], codes[q + 1]), q in [0, n): the node whose
// split (gamma) is q covers the codes that share their first D[q] + 1 bits
// with codes[q], i.e. [a + 1, b], where a is the nearest position left of q
// with a smaller delta and b the nearest one right of q (-1 / n when there is
// none). Its index is a + 1 when D[a] > D[b] (it is its parent's right child)
// and b otherwise (the left child). Inside any node's range the smallest delta
// occurs exactly once, so these are the ranges and splits the reference's
// exact searches find. Only radix node 0 differs: the reference starts it at
// d = 1, l = n - 1 (range [0, n - 1]), so its split is the smallest delta of
// [0, n - 2] and its right end is n - 1. When that is not the overall
// smallest delta (the delta at n - 1 is), the root is "short": node n - 1
// covers the same range and the reference's node 0 writes no children's
// parents.
//
// The parent of node i is the node split at a or b, whichever has the larger
// delta, so the edge count prefix_n[i]/3 - prefix_n[parent[i]]/3
// (kernels/05_edge_count.cpp:3-16) is computed here as well.
//
// Kernels over tiles of 4,096 positions:
//   tree_tiles_kernel     D as bytes and each tile's smallest D, from the
//                         codes (learned build, the C entry);
//   unique_count_kernel,  stage 3 of the whole and batched builds: run heads
//   unique_deltas_kernel  of the sorted keys counted per tile and scanned,
//                         then compacted, each unique code also writing D for
//                         the code before it and the tiles' smallest D (per
//                         cloud in the batched build: tile maps OneKeys /
//                         CloudKeys);
//   tree_nodes_kernel     nearest smaller deltas inside each 32-position
//                         chunk from five ballots over the bits of D (one
//                         lane-parallel table of masks per chunk), across the
//                         tile's chunks from prefix / suffix tables in shared
//                         memory, across tiles (rare: only the tile's running
//                         minima) by a peek at the adjacent tile's edge, then
//                         warp-wide scans of the tile minima and of the found
//                         tile's deltas; then every output of the node split
//                         at each position.
#include <climits>

#include "tree.cuh"

namespace octgb {

constexpr int kTtChunks = kTtTile / 32;
constexpr int kTtAThreads = 256;
constexpr int kTtBThreads = 512;
constexpr int kTtBWarps = kTtBThreads / 32;
constexpr int kTtChunksPerWarp = kTtChunks / kTtBWarps;  // 8
constexpr uint32_t kFull = 0xffffffffu;

static int tt_tiles(int n) { return ((n > 1 ? n : 1) + kTtTile - 1) / kTtTile; }

size_t tree_scratch_bytes_tiles(int tiles) {
  const size_t t = (size_t)(tiles > 1 ? tiles : 1);
  return align_up(t * kTtTile, 256) + align_up(align_up(t, kTtMinBlock), 256) +
         4 * align_up(t * sizeof(int), 256);
}

TreeScratch tree_scratch_carve_tiles(void* base, int tiles) {
  const size_t t = (size_t)(tiles > 1 ? tiles : 1);
  char* p = static_cast<char*>(base);
  TreeScratch S;
  S.tiles = (int)t;
  S.D = reinterpret_cast<uint8_t*>(p);
  p += align_up(t * kTtTile, 256);
  S.tile_min = reinterpret_cast<uint8_t*>(p);
  p += align_up(align_up(t, kTtMinBlock), 256);
  S.tile_sum = reinterpret_cast<int*>(p);
  p += align_up(t * sizeof(int), 256);
  S.tile_prefix = reinterpret_cast<uint32_t*>(p);
  p += align_up(t * sizeof(int), 256);
  S.tile_heads = reinterpret_cast<int*>(p);
  p += align_up(t * sizeof(int), 256);
  S.tile_upos = reinterpret_cast<uint32_t*>(p);
  return S;
}

size_t tree_scratch_bytes(int n) { return tree_scratch_bytes_tiles(tt_tiles(n)); }
TreeScratch tree_scratch_carve(void* base, int n) { return tree_scratch_carve_tiles(base, tt_tiles(n)); }

// Where a tile sits: tiles never cross clouds, and a cloud's tiles start at
// its first position and cover 4,096 positions each; positions are
// cloud-local, arrays are indexed from the cloud's start cs.
struct TileInfo {
  int t;        // tile
  int t_first;  // first and last tile of its cloud
  int t_last;
  int n;        // radix nodes of the cloud
  int lo;       // first position of the tile
  int cs;       // cloud start in the concatenated arrays
};

// One cloud: tile t covers positions [4096 t, 4096 t + 4096).
struct OneCloud {
  int n_host;
  const int* d_unique;
  int tiles;
  __device__ __forceinline__ TileInfo operator()(int t) const {
    TileInfo I;
    I.t = t;
    I.t_first = 0;
    I.t_last = tiles - 1;
    I.n = d_unique ? max(*d_unique - 1, 0) : n_host;
    I.lo = t * kTtTile;
    I.cs = 0;
    return I;
  }
};

// Batched clouds: tile descriptors {first, end, cloud, first tile of cloud}.
struct CloudTiles {
  const int4* tiles;
  const int* start;
  const int* unique_c;
  __device__ __forceinline__ TileInfo operator()(int t) const {
    const int4 d = tiles[t];
    TileInfo I;
    I.t = t;
    I.cs = start[d.z];
    I.t_first = d.w;
    I.t_last = d.w + (start[d.z + 1] - I.cs + kTtTile - 1) / kTtTile - 1;
    I.n = max(unique_c[d.z] - 1, 0);
    I.lo = d.x - I.cs;
    return I;
  }
};

// Delta of cloud position p in the tile-major delta array.
__device__ __forceinline__ size_t d_index(const TileInfo& I, int p) {
  return (size_t)(I.t_first + p / kTtTile) * kTtTile + (size_t)(p % kTtTile);
}

// Lanes whose 5-bit value is below v, from the ballots b[k] of the values'
// bits and v's bits as masks (m[k] all ones where v has bit k).
__device__ __forceinline__ uint32_t lanes_below(const uint32_t (&b)[5], const uint32_t (&m)[5]) {
  uint32_t eq = kFull, lt = 0;
#pragma unroll
  for (int k = 4; k >= 0; --k) {
    lt |= eq & ~b[k] & m[k];
    eq &= ~(b[k] ^ m[k]);
  }
  return lt;
}

__device__ __forceinline__ void bit_masks(uint32_t v, uint32_t (&m)[5]) {
#pragma unroll
  for (int k = 0; k < 5; ++k) m[k] = 0u - ((v >> k) & 1u);
}

__device__ __forceinline__ void value_ballots(uint32_t d, uint32_t (&b)[5]) {
#pragma unroll
  for (int k = 0; k < 5; ++k) b[k] = __ballot_sync(kFull, (d >> k) & 1u);
}


template <class Map>
__global__ void __launch_bounds__(kTtAThreads)
    tree_tiles_kernel(Map map, const uint32_t* __restrict__ codes_all, TreeScratch S) {
  chain_enter();
  constexpr int kWarps = kTtAThreads / 32;
  __shared__ uint32_t s_min[kWarps];
  const TileInfo I = map(blockIdx.x);
  const int n = I.n, t = I.t, t0 = I.lo;
  const uint32_t* codes = codes_all + I.cs;
  uint8_t* Dt = S.D + (size_t)t * kTtTile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (t == 0) {  // whole blocks of the tile-minimum array; the padding never matches
    const int pad = (int)align_up((size_t)S.tiles, kTtMinBlock);
    for (int k = S.tiles + (int)threadIdx.x; k < pad; k += kTtAThreads)
      S.tile_min[k] = (uint8_t)kTtAbsent;
  }
  uint32_t dmin = kTtAbsent;
  if (t0 < n) {
    // a thread takes 4 consecutive positions per step: 16-byte code loads,
    // 4-byte delta stores; the code after the fourth comes from the next lane
    const uint4* c4 = reinterpret_cast<const uint4*>(codes);
    const bool vec = (reinterpret_cast<uintptr_t>(codes) & 15) == 0;
    for (int base = t0 + 4 * (int)threadIdx.x; base < t0 + kTtTile; base += 4 * kTtAThreads) {
      uint32_t c[5];
      if (vec && base + 4 <= n + 1) {
        const uint4 v = c4[base >> 2];
        c[0] = v.x;
        c[1] = v.y;
        c[2] = v.z;
        c[3] = v.w;
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) c[k] = base + k <= n ? codes[base + k] : 0u;
      }
      c[4] = __shfl_down_sync(kFull, c[0], 1);
      if (lane == 31) c[4] = base + 4 <= n ? codes[base + 4] : 0u;
      uint32_t packed = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint32_t d = base + k < n ? tt_delta(c[k], c[k + 1]) : kTtAbsent;
        dmin = min(dmin, d);
        packed |= d << (8 * k);
      }
      *reinterpret_cast<uint32_t*>(Dt + (base - t0)) = packed;
    }
  } else {
    for (int k = threadIdx.x; k < kTtTile / 4; k += kTtAThreads)
      reinterpret_cast<uint32_t*>(Dt)[k] = kTtAbsent * 0x01010101u;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) dmin = min(dmin, __shfl_xor_sync(kFull, dmin, o));
  if (lane == 0) s_min[warp] = dmin;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t m = kTtAbsent;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) m = min(m, s_min[w]);
    S.tile_min[t] = (uint8_t)m;
    S.tile_sum[t] = 0;
  }
}

// Bytes here are at most 31 and so is x: (byte | 0x80) - x keeps the high
// bit exactly when byte >= x, with no borrow between bytes.
__device__ __forceinline__ uint32_t high_bits_below(uint32_t w, uint32_t x4) {
  return ~((w | 0x80808080u) - x4) & 0x80808080u;
}

// Bit j set when byte j of w (16 bytes) is below x.
__device__ __forceinline__ uint32_t bytes_below(const uint4& w, uint32_t x) {
  const uint32_t x4 = x * 0x01010101u;
  const uint32_t v[4] = {w.x, w.y, w.z, w.w};
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    // gather the four high bits (7, 15, 23, 31) into bits 21..24
    const uint32_t h = ((high_bits_below(v[k], x4) >> 7) * 0x00204081u) >> 21;
    m |= (h & 0xFu) << (4 * k);
  }
  return m;
}

// Largest tile in [lo, hi] whose smallest delta is below x, or -1 (whole warp).
__device__ int tiles_scan_left(const uint8_t* __restrict__ tmin, int lo, int hi, uint32_t x,
                               int lane) {
  if (hi < lo) return -1;
  for (int blk = hi / kTtMinBlock; blk >= lo / kTtMinBlock; --blk) {
    const uint4 w = reinterpret_cast<const uint4*>(tmin + (size_t)blk * kTtMinBlock)[lane];
    uint32_t m = bytes_below(w, x);
    const int base = blk * kTtMinBlock + lane * 16;
    if (base > hi || base + 15 < lo) m = 0;
    if (base + 15 > hi && base <= hi) m &= (2u << (hi - base)) - 1u;
    if (base < lo && base + 15 >= lo) m &= ~((1u << (lo - base)) - 1u);
    const uint32_t any = __ballot_sync(kFull, m != 0);
    if (any) {
      const int L = 31 - __clz(any);
      const uint32_t mL = __shfl_sync(kFull, m, L);
      return blk * kTtMinBlock + L * 16 + 31 - __clz(mL);
    }
  }
  return -1;
}

// Smallest tile in [lo, hi] whose smallest delta is below x, or -1 (whole warp).
__device__ int tiles_scan_right(const uint8_t* __restrict__ tmin, int lo, int hi, uint32_t x,
                                int lane) {
  if (hi < lo) return -1;
  for (int blk = lo / kTtMinBlock; blk <= hi / kTtMinBlock; ++blk) {
    const uint4 w = reinterpret_cast<const uint4*>(tmin + (size_t)blk * kTtMinBlock)[lane];
    uint32_t m = bytes_below(w, x);
    const int base = blk * kTtMinBlock + lane * 16;
    if (base > hi || base + 15 < lo) m = 0;
    if (base + 15 > hi && base <= hi) m &= (2u << (hi - base)) - 1u;
    if (base < lo && base + 15 >= lo) m &= ~((1u << (lo - base)) - 1u);
    const uint32_t any = __ballot_sync(kFull, m != 0);
    if (any) {
      const int L = __ffs(any) - 1;
      const uint32_t mL = __shfl_sync(kFull, m, L);
      return blk * kTtMinBlock + L * 16 + __ffs(mL) - 1;
    }
  }
  return -1;
}

// Last (first) position of tile tt's deltas below x; the tile holds one.
__device__ int tile_last_below(const TreeScratch& S, const TileInfo& I, int tt, uint32_t x,
                               int lane) {
  const uint8_t* Dt = S.D + (size_t)tt * kTtTile;
  for (int blk = kTtTile / 512 - 1; blk >= 0; --blk) {
    const uint4 w = reinterpret_cast<const uint4*>(Dt + blk * 512)[lane];
    const uint32_t m = bytes_below(w, x);
    const uint32_t any = __ballot_sync(kFull, m != 0);
    if (any) {
      const int L = 31 - __clz(any);
      const uint32_t mL = __shfl_sync(kFull, m, L);
      return (tt - I.t_first) * kTtTile + blk * 512 + L * 16 + 31 - __clz(mL);
    }
  }
  return -1;
}

__device__ int tile_first_below(const TreeScratch& S, const TileInfo& I, int tt, uint32_t x,
                                int lane) {
  const uint8_t* Dt = S.D + (size_t)tt * kTtTile;
  for (int blk = 0; blk < kTtTile / 512; ++blk) {
    const uint4 w = reinterpret_cast<const uint4*>(Dt + blk * 512)[lane];
    const uint32_t m = bytes_below(w, x);
    const uint32_t any = __ballot_sync(kFull, m != 0);
    if (any) {
      const int L = __ffs(any) - 1;
      const uint32_t mL = __shfl_sync(kFull, m, L);
      // from n on: the last tile's unused tail, so the tile holds no match
      return min((tt - I.t_first) * kTtTile + blk * 512 + L * 16 + __ffs(mL) - 1, I.n);
    }
  }
  return I.n;
}

struct TreeOut {
  uint8_t* prefix_n;
  uint8_t* hll;
  uint8_t* hlr;
  int* left_child;
  int* parent;
  int* ec;  // optional
};

// Radix node 0 as the reference builds it (range [0, n - 1]) with split q.
__device__ __forceinline__ void emit_root(const TreeOut& o, int n, int q, uint32_t x,
                                          bool short_root) {
  const bool ll = q == 0, lr = q + 1 == n - 1;
  o.prefix_n[0] = (uint8_t)x;
  o.left_child[0] = q;
  o.hll[0] = ll;
  o.hlr[0] = lr;
  o.parent[0] = 0;
  if (short_root || lr) o.parent[n - 1] = 0;
  if (!short_root) {
    if (!ll) o.parent[q] = 0;
    if (!lr && q + 1 < n) o.parent[q + 1] = 0;
  }
  if (o.ec) o.ec[0] = 0;
}

template <class Map>
__global__ void __launch_bounds__(kTtBThreads)
    tree_nodes_kernel(Map map, const uint32_t* __restrict__ codes, TreeScratch S, TreeOut o) {
  chain_enter();
  __shared__ __align__(16) uint8_t s_D[kTtTile];
  __shared__ int16_t s_pl[kTtChunks][32];  // last tile position before the chunk with D < v
  __shared__ int16_t s_sf[kTtChunks][32];  // first tile position after the chunk with D < v
  __shared__ int16_t s_wl[kTtBWarps][32], s_wf[kTtBWarps][32];
  __shared__ uint8_t s_pv[kTtTile], s_nv[kTtTile];  // nearest smaller lane in the chunk, or 0xFF
  const TileInfo I = map(blockIdx.x);
  const int n = I.n, t = I.t, t0 = I.lo;
  if (t0 >= n) return;
  // the cloud's arrays
  codes += I.cs;
  o.prefix_n += I.cs;
  o.hll += I.cs;
  o.hlr += I.cs;
  o.left_child += I.cs;
  o.parent += I.cs;
  if (o.ec) o.ec += I.cs;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (n < 2) {  // a single node: the reference's search steps
    if (tid == 0) {
      radix_node(0, n, GlobalCodes{codes}, o.prefix_n, o.hll, o.hlr, o.left_child, o.parent);
      if (o.ec) o.ec[0] = 0;
    }
    return;
  }
  if (tid < kTtTile / 16)
    reinterpret_cast<uint4*>(s_D)[tid] =
        reinterpret_cast<const uint4*>(S.D + (size_t)t * kTtTile)[tid];
  __syncthreads();
  if (t0 + kTtTile > n) {  // the cloud's last tile: positions from n on are absent
    for (int j = n - t0 + tid; j < kTtTile; j += kTtBThreads) s_D[j] = (uint8_t)kTtAbsent;
    __syncthreads();
  }

  const uint32_t below_me = (1u << lane) - 1u;
  const uint32_t above_me = ~below_me << 1;  // lanes > lane (lane 31: none)
  uint32_t lm[5];
  bit_masks((uint32_t)lane, lm);
  int cf[kTtChunksPerWarp];
  int run = -1;
#pragma unroll
  for (int k = 0; k < kTtChunksPerWarp; ++k) {
    const int c = warp * kTtChunksPerWarp + k;
    const uint32_t d = s_D[32 * c + lane];
    uint32_t b[5];
    value_ballots(d, b);
    // lane v: the lanes whose delta is below v; a lane's own query is lane d's
    const uint32_t lt_lane = lanes_below(b, lm);
    const uint32_t lt_own = __shfl_sync(kFull, lt_lane, (int)d);
    const uint32_t l = lt_own & below_me, r = lt_own & above_me;
    s_pv[32 * c + lane] = l ? (uint8_t)(31 - __clz(l)) : (uint8_t)0xFF;
    s_nv[32 * c + lane] = r ? (uint8_t)(__ffs(r) - 1) : (uint8_t)0xFF;
    s_pl[c][lane] = (int16_t)run;
    if (lt_lane) run = 32 * c + 31 - __clz(lt_lane);
    cf[k] = lt_lane ? 32 * c + __ffs(lt_lane) - 1 : kTtTile;
  }
  int runf = kTtTile;
#pragma unroll
  for (int k = kTtChunksPerWarp - 1; k >= 0; --k) {
    const int c = warp * kTtChunksPerWarp + k;
    s_sf[c][lane] = (int16_t)runf;
    runf = min(runf, cf[k]);
  }
  s_wl[warp][lane] = (int16_t)run;
  s_wf[warp][lane] = (int16_t)runf;
  __syncthreads();
  {
    int cl = -1, cr = kTtTile;
    for (int w = 0; w < warp; ++w) cl = max(cl, (int)s_wl[w][lane]);
    for (int w = warp + 1; w < kTtBWarps; ++w) cr = min(cr, (int)s_wf[w][lane]);
#pragma unroll
    for (int k = 0; k < kTtChunksPerWarp; ++k) {
      const int c = warp * kTtChunksPerWarp + k;
      s_pl[c][lane] = (int16_t)max((int)s_pl[c][lane], cl);
      s_sf[c][lane] = (int16_t)min((int)s_sf[c][lane], cr);
    }
  }
  __syncwarp();

  int own_sum = 0;  // edge counts of this tile's nodes emitted here
  // Per chunk, the common case without branches: both neighbours inside the
  // tile (shared-memory tables); lanes needing another tile, the root or an
  // edge count of another tile take warp-uniform guarded blocks.
#pragma unroll 1
  for (int k = 0; k < kTtChunksPerWarp; ++k) {
    const int c = warp * kTtChunksPerWarp + k;
    const int j = 32 * c + lane;
    const int q = t0 + j;
    const bool live = q < n;
    const uint32_t xv = s_D[j];
    const uint32_t pv = s_pv[j], nv = s_nv[j];
    const int pl = s_pl[c][xv], sf = s_sf[c][xv];
    // -2: not in this tile
    int a = pv != 0xFF ? t0 + 32 * c + (int)pv : (pl >= 0 ? t0 + pl : -2);
    int b = nv != 0xFF ? t0 + 32 * c + (int)nv : (sf < kTtTile ? t0 + sf : -2);
    int da = s_D[max(a - t0, 0)], db = s_D[min(max(b - t0, 0), kTtTile - 1)];
    // Neighbours outside the tile (the tile's running minima only): the edge
    // of the adjacent tile first, then one warp-wide scan of the tile minima
    // per query and of the found tile's deltas.
    if (__any_sync(kFull, live && (a == -2 || b == -2))) {
      const bool fa = live && a == -2, fb = live && b == -2;
      if (fa) {
        if (t == I.t_first) {
          a = -1;
        } else {
          const uint4 w = *reinterpret_cast<const uint4*>(S.D + (size_t)t * kTtTile - 16);
          const uint32_t m = bytes_below(w, xv);
          if (m) a = t0 - 16 + 31 - __clz(m);
        }
      }
      if (fb) {
        if (t == I.t_last) {
          b = n;
        } else {
          const uint4 w = *reinterpret_cast<const uint4*>(S.D + (size_t)(t + 1) * kTtTile);
          const uint32_t m = bytes_below(w, xv);
          // a match from n on lies in the last tile's unused tail: none there
          if (m) b = min(t0 + kTtTile + __ffs(m) - 1, n);
        }
      }
      uint32_t need = __ballot_sync(kFull, live && a == -2);
      while (need) {
        const int src = __ffs(need) - 1;
        need &= need - 1;
        const uint32_t qx = __shfl_sync(kFull, xv, src);
        const int tt = tiles_scan_left(S.tile_min, I.t_first, t - 1, qx, lane);
        const int ans = tt >= 0 ? tile_last_below(S, I, tt, qx, lane) : -1;
        if (lane == src) a = ans;
      }
      need = __ballot_sync(kFull, live && b == -2);
      while (need) {
        const int src = __ffs(need) - 1;
        need &= need - 1;
        const uint32_t qx = __shfl_sync(kFull, xv, src);
        const int tt = tiles_scan_right(S.tile_min, t + 1, I.t_last, qx, lane);
        const int ans = tt >= 0 ? tile_first_below(S, I, tt, qx, lane) : n;
        if (lane == src) b = ans;
      }
      if (fa && a >= 0) da = S.D[d_index(I, a)];
      if (fb && b < n) db = S.D[d_index(I, b)];
    }
    if (a < 0) da = -1;
    if (b >= n) db = -1;
    // a < 0 and b >= n: the smallest delta overall (the proper root), which
    // gives radix node 0 unless it sits at n - 1 (a short root: node 0 then
    // comes from the split of [0, n - 2], with a < 0 and b == n - 1).
    const bool top = a < 0 && b >= n;
    const bool short_root = a < 0 && b == n - 1;
    if (live && !top) {
      const int i = a < 0 ? b : (b >= n ? a + 1 : (da > db ? a + 1 : b));
      const bool ll = a + 1 == q, lr = b == q + 1;
      o.prefix_n[i] = (uint8_t)xv;
      o.left_child[i] = q;
      o.hll[i] = ll;
      o.hlr[i] = lr;
      if (!ll) o.parent[q] = i;
      if (!lr) o.parent[q + 1] = i;
      if (o.ec) {
        // the larger neighbour delta is the parent's (>= 0 whenever read)
        const int e = short_root ? 0 : (int)(xv / 3u) - (int)((uint32_t)max(da, db) / 3u);
        o.ec[i] = e;
        const int ti = I.t_first + i / kTtTile;
        own_sum += ti == t ? e : 0;
        if (ti != t) atomicAdd(S.tile_sum + ti, e);
      }
    }
    if (__any_sync(kFull, live && (top || short_root))) {
      if (live && top && q <= n - 2) emit_root(o, n, q, xv, false);
      if (live && short_root) emit_root(o, n, q, xv, true);
    }
  }
  if (o.ec) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) own_sum += __shfl_xor_sync(kFull, own_sum, off);
    if (lane == 0 && own_sum != 0) atomicAdd(S.tile_sum + t, own_sum);
  }
}

// ------------------------------------------------------ unique + deltas --
constexpr int kUdThreads = 256;
constexpr int kUdItems = kTtTile / kUdThreads;  // 16

__device__ __forceinline__ int ud_pad(int j) { return j + (j >> 5); }

// A 4,096-key tile of sorted keys: keys [lo, hi) of the cloud starting at cs,
// whose unique codes go to the tree tiles from t_first on.
struct KeyTile {
  int lo, hi, cs, t_first, cloud;
  bool last;  // the cloud's last tile
};

// One cloud of n keys.
struct OneKeys {
  int n;
  __device__ __forceinline__ KeyTile operator()(int t) const {
    KeyTile K;
    K.lo = t * kTtTile;
    K.hi = min(K.lo + kTtTile, n);
    K.cs = 0;
    K.t_first = 0;
    K.cloud = 0;
    K.last = K.hi >= n;
    return K;
  }
};

// Batched clouds: tile descriptors {first, end, cloud, first tile of cloud}.
struct CloudKeys {
  const int4* tiles;
  int n_tiles;
  const int* start;
  __device__ __forceinline__ KeyTile operator()(int t) const {
    const int4 d = tiles[t];
    KeyTile K;
    K.lo = d.x;
    K.hi = d.y;
    K.cs = start[d.z];
    K.t_first = d.w;
    K.cloud = d.z;
    K.last = t == n_tiles - 1 || tiles[t + 1].z != d.z;
    return K;
  }
};

// Run heads of sorted keys per tile; also resets the tree tiles' edge-count
// sums and smallest deltas.
template <class Map>
__global__ void __launch_bounds__(kUdThreads)
    unique_count_kernel(const uint32_t* __restrict__ keys, Map map, int n_tiles, TreeScratch S,
                        const uint32_t* __restrict__ gate) {
  chain_enter();
  if (gate && *gate == 0) return;
  __shared__ int s_cnt[kUdThreads / 32];
  const int tid = threadIdx.x;
  // CTAs walk the tiles (a capped grid: a gated-off launch schedules few CTAs)
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const KeyTile K = map(t);
    if (t == 0) {
      const int pad = (int)align_up((size_t)S.tiles, kTtMinBlock);
      for (int k = S.tiles + tid; k < pad; k += kUdThreads) S.tile_min[k] = (uint8_t)kTtAbsent;
    }
    if (tid == 0) {
      S.tile_min[t] = (uint8_t)kTtAbsent;
      S.tile_sum[t] = 0;
    }
    int cnt = 0;
    const int j0 = K.lo + tid * kUdItems;
    if ((reinterpret_cast<uintptr_t>(keys + K.lo) & 15) != 0) {
      // Unaligned tile (a cloud starting mid-vector): warp-striped loads of
      // each key and the one before it, coalesced, instead of 16 scalar
      // strided loads per thread.
#pragma unroll 4
      for (int q = 0; q < kUdItems; ++q) {
        const int j = K.lo + q * kUdThreads + tid;
        if (j < K.hi) {
          const uint32_t k = keys[j];
          cnt += (j == K.cs) || k != keys[j - 1];
        }
      }
    } else if (j0 < K.hi) {
      uint32_t prev = j0 > K.cs ? keys[j0 - 1] : 0u;
      uint32_t k[kUdItems];
      if (j0 + kUdItems <= K.hi && (reinterpret_cast<uintptr_t>(keys + j0) & 15) == 0) {
#pragma unroll
        for (int q = 0; q < kUdItems / 4; ++q) {
          const uint4 v = reinterpret_cast<const uint4*>(keys + j0)[q];
          k[4 * q] = v.x;
          k[4 * q + 1] = v.y;
          k[4 * q + 2] = v.z;
          k[4 * q + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int q = 0; q < kUdItems; ++q) k[q] = j0 + q < K.hi ? keys[j0 + q] : 0u;
      }
#pragma unroll
      for (int q = 0; q < kUdItems; ++q) {
        if (j0 + q < K.hi) {
          cnt += (j0 + q == K.cs) || k[q] != prev;
          prev = k[q];
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o);
    if ((tid & 31) == 0) s_cnt[tid >> 5] = cnt;
    __syncthreads();
    if (tid == 0) {
      int total = 0;
      for (int w = 0; w < kUdThreads / 32; ++w) total += s_cnt[w];
      S.tile_heads[t] = total;
    }
    __syncthreads();  // s_cnt is the next tile's
  }
}

// Compaction from the tile prefixes; each unique code at (cloud) position
// o >= 1 also writes D[o - 1], the delta to the code before it (the last key
// of the previous run), and the tiles' smallest deltas. With unique_c, each
// cloud's last tile writes the cloud's U.
template <class Map>
__global__ void __launch_bounds__(kUdThreads)
    unique_deltas_kernel(const uint32_t* __restrict__ keys, Map map, uint32_t* __restrict__ out,
                         int n_tiles, TreeScratch S, int* __restrict__ unique_c,
                         const uint32_t* __restrict__ gate) {
  chain_enter();
  if (gate && *gate == 0) return;
  __shared__ uint32_t s_keys[kTtTile + kTtTile / 32];
  __shared__ uint8_t s_d[kTtTile];
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  __shared__ uint32_t s_min[2][kUdThreads / 32];
  const int tid = threadIdx.x;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const KeyTile K = map(t);
    const int valid = K.hi - K.lo;
    if (valid <= 0) continue;  // uniform in the CTA
#pragma unroll 4
    for (int j = tid; j < kTtTile; j += kUdThreads) {
      const int idx = K.lo + j;
      s_keys[ud_pad(j)] = j < valid ? keys[idx] : 0u;
    }
    const uint32_t before = K.lo > K.cs ? keys[K.lo - 1] : 0u;
    __syncthreads();
    uint32_t key[kUdItems], dk[kUdItems];
    uint32_t flags = 0;
    int cnt = 0;
    const int j0 = tid * kUdItems;
    uint32_t prev = j0 == 0 ? before : s_keys[ud_pad(j0 - 1)];
#pragma unroll
    for (int k = 0; k < kUdItems; ++k) {
      key[k] = s_keys[ud_pad(j0 + k)];
      const int j = j0 + k;
      const bool head = j < valid && ((K.lo + j == K.cs) || key[k] != prev);
      dk[k] = tt_delta(prev, key[k]);  // used for heads past the cloud's first code only
      flags |= (uint32_t)head << k;
      cnt += head;
      prev = key[k];
    }
    const uint32_t off = block_exclusive_sum<kUdThreads>((uint32_t)cnt, s_warp, &s_total);
    const uint32_t total = s_total;
    const uint32_t base = S.tile_upos[t] - S.tile_upos[K.t_first];
    // Stage the heads (s_keys is free after the scan's barriers) and their deltas.
    uint32_t o = off;
#pragma unroll
    for (int k = 0; k < kUdItems; ++k) {
      if (flags >> k & 1u) {
        s_keys[ud_pad(o)] = key[k];
        s_d[o] = (uint8_t)dk[k];
        ++o;
      }
    }
    __syncthreads();
    // Deltas go to positions base - 1 .. base + total - 2 (the cloud's first code
    // has none), i.e. the cloud's tree tiles ta and at most ta + 1.
    const int first = base == 0 ? 1 : 0;
    const int ta = (int)(base + first - 1) / kTtTile;
    uint32_t ma = kTtAbsent, mb = kTtAbsent;
    for (int j = tid; j < (int)total; j += kUdThreads) {
      out[K.cs + base + j] = s_keys[ud_pad(j)];
      if (j >= first) {
        const int pos = (int)base + j - 1;
        const uint32_t d = s_d[j];
        S.D[(size_t)(K.t_first + pos / kTtTile) * kTtTile + pos % kTtTile] = (uint8_t)d;
        if (pos / kTtTile == ta) ma = min(ma, d);
        else mb = min(mb, d);
      }
    }
#pragma unroll
    for (int sh = 16; sh > 0; sh >>= 1) {
      ma = min(ma, __shfl_xor_sync(kFull, ma, sh));
      mb = min(mb, __shfl_xor_sync(kFull, mb, sh));
    }
    if ((tid & 31) == 0) {
      s_min[0][tid >> 5] = ma;
      s_min[1][tid >> 5] = mb;
    }
    __syncthreads();
    if (tid == 0) {
      if ((int)total > first) {
        uint32_t a = kTtAbsent, b = kTtAbsent;
        for (int w = 0; w < kUdThreads / 32; ++w) {
          a = min(a, s_min[0][w]);
          b = min(b, s_min[1][w]);
        }
        if (a < kTtAbsent) atomic_min_u8(S.tile_min + K.t_first + ta, a);
        if (b < kTtAbsent) atomic_min_u8(S.tile_min + K.t_first + ta + 1, b);
      }
      if (unique_c && K.last) unique_c[K.cloud] = (int)(base + total);
    }
    __syncthreads();  // the shared arrays are the next tile's
  }
}

// Grid of the whole build's (gated) unique kernels: the tiles, capped at 8
// CTAs per SM.
static int unique_grid(int tiles) {
  const int cap = device_sm_count() * 8;
  return tiles < cap ? tiles : cap;
}

cudaError_t launch_unique_deltas(const uint32_t* sorted, int n, uint32_t* codes_out, int* d_unique,
                                 void* tree_scratch, cudaStream_t s, const uint32_t* gate) {
  if (n <= 0) return cudaMemsetAsync(d_unique, 0, sizeof(int), s);
  const TreeScratch S = tree_scratch_carve(tree_scratch, n);
  const OneKeys map{n};
  cudaError_t e = launch_chained(unique_count_kernel<OneKeys>, dim3(unique_grid(S.tiles)),
                                 dim3(kUdThreads), 0, s, sorted, map, S.tiles, S, gate);
  if (e == cudaSuccess)
    e = launch_tile_counts_scan(S.tiles, S.tile_heads, S.tile_upos, d_unique, s, gate);
  if (e != cudaSuccess) return e;
  return launch_chained(unique_deltas_kernel<OneKeys>, dim3(unique_grid(S.tiles)), dim3(kUdThreads),
                        0, s, sorted, map, codes_out, S.tiles, S, nullptr, gate);
}

cudaError_t launch_batch_unique_deltas(const uint32_t* sorted, const int4* tiles, int n_tiles,
                                       const int* start, uint32_t* codes_out, int* unique_c,
                                       void* scratch, cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  const TreeScratch S = tree_scratch_carve_tiles(scratch, n_tiles);
  const CloudKeys map{tiles, n_tiles, start};
  cudaError_t e = launch_chained(unique_count_kernel<CloudKeys>, dim3(n_tiles), dim3(kUdThreads), 0,
                                 s, sorted, map, n_tiles, S, nullptr);
  if (e == cudaSuccess) e = launch_tile_counts_scan(n_tiles, S.tile_heads, S.tile_upos, nullptr, s);
  if (e != cudaSuccess) return e;
  return launch_chained(unique_deltas_kernel<CloudKeys>, dim3(n_tiles), dim3(kUdThreads), 0, s,
                        sorted, map, codes_out, n_tiles, S, unique_c, nullptr);
}

cudaError_t launch_batch_radix_tree_from_deltas(const int4* tiles, int n_tiles, const int* start,
                                                const int* unique_c, const uint32_t* codes,
                                                uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                                                int* left_child, int* parent, int* ec,
                                                void* scratch, cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  const TreeScratch S = tree_scratch_carve_tiles(scratch, n_tiles);
  const CloudTiles map{tiles, start, unique_c};
  const TreeOut o{prefix_n, hll, hlr, left_child, parent, ec};
  return launch_chained(tree_nodes_kernel<CloudTiles>, dim3(n_tiles), dim3(kTtBThreads), 0, s, map,
                        codes, S, o);
}

cudaError_t launch_radix_tree_from_deltas(int n_host, const int* d_unique, const uint32_t* codes,
                                          uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                                          int* left_child, int* parent, int* ec, void* scratch,
                                          cudaStream_t s) {
  if (n_host <= 0) return cudaSuccess;
  const TreeScratch S = tree_scratch_carve(scratch, n_host);
  const OneCloud map{n_host, d_unique, S.tiles};
  const TreeOut o{prefix_n, hll, hlr, left_child, parent, ec};
  return launch_chained(tree_nodes_kernel<OneCloud>, dim3(S.tiles), dim3(kTtBThreads), 0, s, map,
                        codes, S, o);
}

cudaError_t launch_radix_tree_sorted(int n_host, const int* d_unique, const uint32_t* codes,
                                     uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                                     int* left_child, int* parent, int* ec, void* scratch,
                                     cudaStream_t s) {
  if (n_host <= 0) return cudaSuccess;
  const TreeScratch S = tree_scratch_carve(scratch, n_host);
  const OneCloud map{n_host, d_unique, S.tiles};
  cudaError_t e = launch_chained(tree_tiles_kernel<OneCloud>, dim3(S.tiles), dim3(kTtAThreads), 0,
                                 s, map, codes, S);
  if (e != cudaSuccess) return e;
  const TreeOut o{prefix_n, hll, hlr, left_child, parent, ec};
  return launch_chained(tree_nodes_kernel<OneCloud>, dim3(S.tiles), dim3(kTtBThreads), 0, s, map,
                        codes, S, o);
}

cudaError_t launch_batch_radix_tree(const int4* tiles, int n_tiles, const int* start,
                                    const int* unique_c, const uint32_t* codes, uint8_t* prefix_n,
                                    uint8_t* hll, uint8_t* hlr, int* left_child, int* parent,
                                    int* ec, void* scratch, cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  const TreeScratch S = tree_scratch_carve_tiles(scratch, n_tiles);
  const CloudTiles map{tiles, start, unique_c};
  cudaError_t e = launch_chained(tree_tiles_kernel<CloudTiles>, dim3(n_tiles), dim3(kTtAThreads), 0,
                                 s, map, codes, S);
  if (e != cudaSuccess) return e;
  const TreeOut o{prefix_n, hll, hlr, left_child, parent, ec};
  return launch_chained(tree_nodes_kernel<CloudTiles>, dim3(n_tiles), dim3(kTtBThreads), 0, s, map,
                        codes, S, o);
}

}  // namespace octgb
