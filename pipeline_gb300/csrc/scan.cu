// Stage 3 (unique) and stages 5-6 (edge count + inclusive prefix sum).
//
// The stage entry points are single-pass tile scans with decoupled look-back:
// a tile takes the next id from an atomic counter, reduces its items,
// publishes its aggregate, waits (bounded) for the inclusive prefix of the
// tiles before it and writes. The whole builds take the tile prefixes from a
// scan of per-tile sums made earlier (run heads: csrc/tree_tiled.cu; edge
// counts: the tree kernel), so their tiles never wait on one another.
//
// Unique replaces k_CountUnique (reference include/kernels/03_unique.hpp:4,
// kernels/03_unique.cpp:2-16; the reference GPU form is one thread,
// kernels/cuda/03_unique.cu:5-24). It may run in place: every output position
// is at or before its input position, and a tile writes only after the tiles
// before it published their aggregates, which they do after loading.
//
// Edge count + prefix sum replace k_EdgeCount
// (include/kernels/05_edge_count.hpp:5-8) and k_PartialSum
// (include/kernels/06_partial_sum.hpp:6-9; the reference GPU driver does this
// scan on the host, apps/gpu_demo/main.cu:308-310). Fused, one read of
// prefix_n/parent produces both arrays and the octree node count.
#include "tree.cuh"

namespace octgb {

constexpr unsigned long long kLbAgg = 1ull << 62;
constexpr unsigned long long kLbInc = 2ull << 62;
constexpr unsigned long long kLbFlags = 3ull << 62;

// One full warp per tile: lane l probes predecessor (pred - l) with a relaxed
// load (flag and value share a 64-bit word), so one round trip covers 32
// predecessors. Returns the exclusive prefix in every lane; lane 0 publishes.
__device__ uint32_t warp_lookback_u32(unsigned long long* lb, int tile, uint32_t agg,
                                      uint32_t* status,
                                      unsigned long long limit_ns = kWaitLimitNs) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) st_release_u64(lb, kLbInc | agg);
    return 0;
  }
  if (lane == 0) st_release_u64(lb + tile, kLbAgg | agg);
  uint32_t ex = 0;
  int pred = tile - 1;
  WaitBound wait(limit_ns);
  while (true) {
    const int p = pred - lane;
    const unsigned long long w = p >= 0 ? ld_relaxed_u64(lb + p) : kLbInc;
    const unsigned long long f = w & kLbFlags;
    const uint32_t inc_m = __ballot_sync(0xffffffffu, f == kLbInc);
    const uint32_t nr_m = __ballot_sync(0xffffffffu, f == 0);
    const int first_inc = inc_m ? __ffs(inc_m) - 1 : 32;
    const int first_nr = nr_m ? __ffs(nr_m) - 1 : 32;
    if (first_nr < first_inc) {  // take the ready words before it, wait on it
      ex += __reduce_add_sync(0xffffffffu, lane < first_nr ? (uint32_t)w : 0u);
      pred -= first_nr;
      if (__any_sync(0xffffffffu, wait.expired())) {  // the warp leaves together
        if (lane == 0) raise_status(status, kStatusSpinTimeout);
        break;
      }
      continue;
    }
    const int take = first_inc < 32 ? first_inc + 1 : 32;
    ex += __reduce_add_sync(0xffffffffu, lane < take ? (uint32_t)w : 0u);
    if (first_inc < 32) break;
    pred -= 32;
  }
  if (lane == 0) st_release_u64(lb + tile, kLbInc | (uint32_t)(ex + agg));
  return ex;
}

// Diagnostics: the warp look-back of tile 1 whose predecessor (tile 0) never
// publishes; it must give up after limit_ns with the status bit set.
__global__ void diag_warp_wait_kernel(unsigned long long* lb, uint32_t* status,
                                      unsigned long long limit_ns) {
  warp_lookback_u32(lb, 1, 1u, status, limit_ns);
}

cudaError_t launch_diag_scan_wait(unsigned long long* lb, uint32_t* status,
                                  unsigned long long limit_ns, cudaStream_t s) {
  diag_warp_wait_kernel<<<1, 32, 0, s>>>(lb, status, limit_ns);
  return cudaGetLastError();
}

// --------------------------------------------------------------------------
// Unique.
// --------------------------------------------------------------------------
constexpr int kUqThreads = 256;
constexpr int kUqItems = 16;
constexpr int kUqTile = kUqThreads * kUqItems;

__device__ __forceinline__ int pad_idx(int j) { return j + (j >> 5); }

__global__ void __launch_bounds__(kUqThreads)
    unique_kernel(const uint32_t* src, uint32_t* dst, int n, int* __restrict__ d_count,
                  unsigned long long* __restrict__ lb, uint32_t* __restrict__ counter, int tiles,
                  uint32_t* __restrict__ status, const uint32_t* __restrict__ gate) {
  chain_enter();
  if (gate && *gate == 0) return;
  __shared__ uint32_t s_keys[kUqTile + kUqTile / 32];
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_misc[4];
  const int tid = threadIdx.x;
  if (tid == 0) s_misc[0] = atomicAdd(counter, 1u);
  __syncthreads();
  const int tile = (int)s_misc[0];
  const int start = tile * kUqTile;
  const int valid = min(kUqTile, n - start);
  // Coalesced load into padded shared memory (plus the key before the tile).
#pragma unroll 4
  for (int j = tid; j < kUqTile; j += kUqThreads) {
    const int idx = start + j;
    s_keys[pad_idx(j)] = idx < n ? src[idx] : 0u;
  }
  uint32_t before = 0;
  if (tid == 0 && start > 0) before = src[start - 1];
  if (tid == 0) s_misc[1] = before;
  __syncthreads();
  // Blocked flags: item j = tid * ITEMS + k is a run head if it differs from j - 1.
  uint32_t key[kUqItems];
  uint32_t flags = 0;
  int cnt = 0;
  const int j0 = tid * kUqItems;
  uint32_t prev = j0 == 0 ? s_misc[1] : s_keys[pad_idx(j0 - 1)];
#pragma unroll
  for (int k = 0; k < kUqItems; ++k) {
    key[k] = s_keys[pad_idx(j0 + k)];
    const int j = j0 + k;
    const bool head = j < valid && ((start + j == 0) || key[k] != prev);
    flags |= (uint32_t)head << k;
    cnt += head;
    prev = key[k];
  }
  uint32_t total;
  const uint32_t off = block_exclusive_sum<kUqThreads>((uint32_t)cnt, s_warp, &s_misc[2]);
  total = s_misc[2];
  if (tid < 32) {
    const uint32_t e = warp_lookback_u32(lb, tile, total, status);
    if (tid == 0) s_misc[3] = e;
  }
  // Stage the tile's run heads contiguously (s_keys is free after the scan's barriers).
  uint32_t o = off;
#pragma unroll
  for (int k = 0; k < kUqItems; ++k)
    if (flags >> k & 1u) s_keys[pad_idx(o++)] = key[k];
  __syncthreads();
  const uint32_t ex = s_misc[3];
  for (int j = tid; j < (int)total; j += kUqThreads) dst[ex + j] = s_keys[pad_idx(j)];
  if (tid == 0 && tile == tiles - 1) *d_count = (int)(ex + total);
}

ScanPlan unique_plan(int n) {
  ScanPlan p{};
  p.n = n;
  p.tile = kUqTile;
  p.tiles = n > 0 ? (n + kUqTile - 1) / kUqTile : 0;
  p.counter_off = 0;
  p.lookback_off = 256;
  p.bytes = align_up(p.lookback_off + sizeof(unsigned long long) * (size_t)(p.tiles + 1), 256);
  return p;
}

cudaError_t launch_unique_gated(const uint32_t* src, uint32_t* dst, int n, int* d_count,
                                const ScanPlan* plan, void* ctrl, uint32_t* status,
                                const uint32_t* gate, cudaStream_t s) {
  if (n <= 0) return gate ? cudaSuccess : cudaMemsetAsync(d_count, 0, sizeof(int), s);
  char* c = static_cast<char*>(ctrl);
  return launch_chained(unique_kernel, dim3(plan->tiles), dim3(kUqThreads), 0, s, src, dst, n,
                        d_count, reinterpret_cast<unsigned long long*>(c + plan->lookback_off),
                        reinterpret_cast<uint32_t*>(c + plan->counter_off), plan->tiles, status,
                        gate);
}

cudaError_t launch_unique(const uint32_t* src, uint32_t* dst, int n, int* d_count,
                          const ScanPlan* plan, void* ctrl, uint32_t* status, cudaStream_t s) {
  return launch_unique_gated(src, dst, n, d_count, plan, ctrl, status, nullptr, s);
}

// --------------------------------------------------------------------------
// Edge count + inclusive prefix sum.
// --------------------------------------------------------------------------
constexpr int kEsThreads = 256;
constexpr int kEsItems = 16;
constexpr int kEsTile = kEsThreads * kEsItems;

__global__ void __launch_bounds__(kEsThreads)
    edge_scan_kernel(int mode, int n_host, const int* __restrict__ d_unique,
                     const uint8_t* __restrict__ prefix_n, const int* __restrict__ parent,
                     int* ec_out, int* __restrict__ ps_out, int* __restrict__ d_max_slot,
                     unsigned long long* __restrict__ lb, uint32_t* __restrict__ counter,
                     uint32_t* __restrict__ status, OctTags zt,
                     const uint32_t* __restrict__ tile_prefix) {
  chain_enter();
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_misc[4];
  __shared__ int s_max[kEsThreads / 32];
  __shared__ int s_hi;
  const int n = d_unique ? max(*d_unique - 1, 0) : n_host;
  const int tid = threadIdx.x;
  // Edge count alone has no cross-tile dependency: the block index is the tile.
  if (tid == 0)
    s_misc[0] = (mode == kEdgeOnly || tile_prefix) ? blockIdx.x : atomicAdd(counter, 1u);
  __syncthreads();
  const int tile = (int)s_misc[0];
  const int start = tile * kEsTile;
  if (start >= n) return;  // tiles past the end: nobody waits on them
  const int tiles = (n + kEsTile - 1) / kEsTile;
  const int j0 = start + tid * kEsItems;

  int v[kEsItems];
  // A thread's 16 items are contiguous: 128-bit loads when in range and aligned.
  const bool vec = j0 + kEsItems <= n &&
                   ((reinterpret_cast<uintptr_t>(prefix_n) | reinterpret_cast<uintptr_t>(parent) |
                     reinterpret_cast<uintptr_t>(ec_out) | reinterpret_cast<uintptr_t>(ps_out)) &
                    15u) == 0;
  if (mode & kEdgeOnly) {
    int par[kEsItems];
    uint8_t pn[kEsItems];
    if (vec) {
      const uint4 pb = *reinterpret_cast<const uint4*>(prefix_n + j0);
      const uint32_t pw[4] = {pb.x, pb.y, pb.z, pb.w};
#pragma unroll
      for (int k = 0; k < kEsItems; ++k) pn[k] = (uint8_t)(pw[k >> 2] >> (8 * (k & 3)));
#pragma unroll
      for (int q = 0; q < kEsItems / 4; ++q) {
        const int4 t = *reinterpret_cast<const int4*>(parent + j0 + 4 * q);
        par[4 * q] = t.x;
        par[4 * q + 1] = t.y;
        par[4 * q + 2] = t.z;
        par[4 * q + 3] = t.w;
      }
    } else {
#pragma unroll
      for (int k = 0; k < kEsItems; ++k) {
        const int i = j0 + k;
        pn[k] = i < n ? prefix_n[i] : 0;
        par[k] = i < n ? parent[i] : 0;
      }
    }
#pragma unroll
    for (int k = 0; k < kEsItems; ++k) {
      const int i = j0 + k;
      int e = 0;
      if (i > 0 && i < n) {
        int p = par[k];
        if ((unsigned)p >= (unsigned)n) {  // malformed input: never read out of bounds
          raise_status(status, kStatusWalkLimit);
          p = 0;
        }
        e = (int)(pn[k] / 3) - (int)(prefix_n[p] / 3);
      }
      v[k] = e;
    }
    if (!(mode & kScanOnly)) {
      if (vec) {
#pragma unroll
        for (int q = 0; q < kEsItems / 4; ++q)
          *reinterpret_cast<int4*>(ec_out + j0 + 4 * q) =
              make_int4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      } else {
#pragma unroll
        for (int k = 0; k < kEsItems; ++k)
          if (j0 + k < n) ec_out[j0 + k] = v[k];
      }
      return;
    }
  } else if (vec) {
#pragma unroll
    for (int q = 0; q < kEsItems / 4; ++q) {
      const int4 t = *reinterpret_cast<const int4*>(ec_out + j0 + 4 * q);
      v[4 * q] = t.x;
      v[4 * q + 1] = t.y;
      v[4 * q + 2] = t.z;
      v[4 * q + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kEsItems; ++k) v[k] = j0 + k < n ? ec_out[j0 + k] : 0;
  }
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kEsItems; ++k) sum += (uint32_t)v[k];
  const uint32_t off = block_exclusive_sum<kEsThreads>(sum, s_warp, &s_misc[2]);
  if (tile_prefix) {  // tile prefixes known in advance
    if (tid == 0) s_misc[3] = tile_prefix[tile];
  } else if (tid < 32) {
    const uint32_t e = warp_lookback_u32(lb, tile, s_misc[2], status);
    if (tid == 0) s_misc[3] = e;
  }
  __syncthreads();
  uint32_t run = s_misc[3] + off;
  int mx = 0;
  int ps[kEsItems];
#pragma unroll
  for (int k = 0; k < kEsItems; ++k) {
    const int i = j0 + k;
    run += (uint32_t)v[k];
    ps[k] = (int)run;
    if (i < n) {
      const int last = v[k] > 0 ? (int)run + v[k] - 1 : (int)run;
      if (i > 0 && v[k] > 0 && last > mx) mx = last;
      if (i == n - 1 && (int)run > mx) mx = (int)run;
    }
  }
  if (vec) {
#pragma unroll
    for (int q = 0; q < kEsItems / 4; ++q) {
      if (mode == kEdgeAndScan)
        *reinterpret_cast<int4*>(ec_out + j0 + 4 * q) =
            make_int4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      *reinterpret_cast<int4*>(ps_out + j0 + 4 * q) =
          make_int4(ps[4 * q], ps[4 * q + 1], ps[4 * q + 2], ps[4 * q + 3]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < kEsItems; ++k) {
      const int i = j0 + k;
      if (i < n) {
        if (mode == kEdgeAndScan) ec_out[i] = v[k];
        ps_out[i] = ps[k];
      }
    }
  }
  if (d_max_slot || zt.child) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) s_max[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
      int m = 0;
      for (int w = 0; w < kEsThreads / 32; ++w) m = max(m, s_max[w]);
      if (d_max_slot) atomicMax(d_max_slot, m);
      // The tile's octree slots: from its exclusive prefix (the slot after the
      // previous tile's last prefix) to its largest slot or its last prefix.
      s_hi = max(m, (int)(s_misc[3] + s_misc[2]));
    }
  }
  if (zt.child) {
    // Clear the octree tags of those slots (the intervals of consecutive tiles
    // meet, so all of [0, M) is cleared before stages 7-8 run).
    __syncthreads();
    const int lo = (int)s_misc[3];
    const int hi = min(s_hi, zt.cap - 1);
    if (hi >= lo) clear_tag_range(zt, (size_t)lo, (size_t)hi, tid, kEsThreads);
  }
  (void)tiles;
}

ScanPlan edge_scan_plan(int n) {
  ScanPlan p{};
  p.n = n;
  p.tile = kEsTile;
  p.tiles = n > 0 ? (n + kEsTile - 1) / kEsTile : 0;
  p.counter_off = 0;
  p.lookback_off = 256;
  p.bytes = align_up(p.lookback_off + sizeof(unsigned long long) * (size_t)(p.tiles + 1), 256);
  return p;
}

cudaError_t launch_edge_scan(int mode, int n_host, const int* d_unique, const uint8_t* prefix_n,
                             const int* parent, int* ec, int* ps, int* d_max_slot,
                             const ScanPlan* plan, void* ctrl, uint32_t* status, cudaStream_t s) {
  if (plan->tiles <= 0) return cudaSuccess;
  char* c = static_cast<char*>(ctrl);
  unsigned long long* lb =
      c ? reinterpret_cast<unsigned long long*>(c + plan->lookback_off) : nullptr;
  uint32_t* counter = c ? reinterpret_cast<uint32_t*>(c + plan->counter_off) : nullptr;
  if (mode != kEdgeOnly && !c) return cudaErrorInvalidValue;
  return launch_chained(edge_scan_kernel, dim3(plan->tiles), dim3(kEsThreads), 0, s, mode, n_host,
                        d_unique, prefix_n, parent, ec, ps, d_max_slot, lb, counter, status,
                        OctTags{}, nullptr);
}

// Exclusive scan of the per-tile edge-count sums (one CTA).
constexpr int kTsThreads = 1024;
__global__ void __launch_bounds__(kTsThreads)
    tile_sums_scan_kernel(int tiles_fixed, int n_host, const int* __restrict__ d_unique,
                          const int* __restrict__ tile_sum, uint32_t* __restrict__ tile_prefix,
                          int* __restrict__ total_out, const uint32_t* __restrict__ gate) {
  chain_enter();
  if (gate && *gate == 0) return;
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  const int n = d_unique ? max(*d_unique - 1, 0) : n_host;
  const int tiles = tiles_fixed > 0 ? tiles_fixed : (n + kEsTile - 1) / kEsTile;
  const int per = (tiles + kTsThreads - 1) / kTsThreads;
  const int j0 = threadIdx.x * per;
  uint32_t sum = 0;
  for (int j = j0; j < min(j0 + per, tiles); ++j) sum += (uint32_t)tile_sum[j];
  uint32_t run = block_exclusive_sum<kTsThreads>(sum, s_warp, &s_total);
  for (int j = j0; j < min(j0 + per, tiles); ++j) {
    tile_prefix[j] = run;
    run += (uint32_t)tile_sum[j];
  }
  if (total_out && threadIdx.x == 0) *total_out = (int)s_total;
}

cudaError_t launch_prefix_sum_clear_tags(int n_host, const int* d_unique, int* ec, int* ps,
                                         int* d_max_slot, void* tree_scratch, uint32_t* status,
                                         const OctTags& tags, cudaStream_t s) {
  static_assert(kEsTile == 4096, "scan tiles are the radix-tree tiles");
  if (n_host <= 0) return cudaSuccess;
  const TreeScratch S = tree_scratch_carve(tree_scratch, n_host);
  cudaError_t e = launch_chained(tile_sums_scan_kernel, dim3(1), dim3(kTsThreads), 0, s, 0, n_host,
                                 d_unique, S.tile_sum, S.tile_prefix, nullptr, nullptr);
  if (e != cudaSuccess) return e;
  const int tiles = (n_host + kEsTile - 1) / kEsTile;
  return launch_chained(edge_scan_kernel, dim3(tiles), dim3(kEsThreads), 0, s, kScanOnly, n_host,
                        d_unique, nullptr, nullptr, ec, ps, d_max_slot, nullptr, nullptr, status,
                        tags.cap > 0 ? tags : OctTags{}, S.tile_prefix);
}

__global__ void __launch_bounds__(256)
    radix_tree_kernel(int n_host, const int* __restrict__ d_unique,
                      const uint32_t* __restrict__ codes, uint8_t* __restrict__ prefix_n,
                      uint8_t* __restrict__ hll, uint8_t* __restrict__ hlr,
                      int* __restrict__ left_child, int* __restrict__ parent) {
  chain_enter();
  const int n = d_unique ? max(*d_unique - 1, 0) : n_host;
  const int stride = gridDim.x * blockDim.x;
  const GlobalCodes gc{codes};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    radix_node(i, n, gc, prefix_n, hll, hlr, left_child, parent);
}

cudaError_t launch_radix_tree(int n_host, const int* d_unique, const uint32_t* codes,
                              uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr, int* left_child,
                              int* parent, cudaStream_t s) {
  if (n_host <= 0) return cudaSuccess;
  const int grid = (n_host + 255) / 256;
  return launch_chained(radix_tree_kernel, dim3(grid), dim3(256), 0, s, n_host, d_unique, codes,
                        prefix_n, hll, hlr, left_child, parent);
}

cudaError_t launch_tile_sums_scan(int tiles, const int* tile_sum, uint32_t* tile_prefix,
                                  cudaStream_t s) {
  if (tiles <= 0) return cudaSuccess;
  return launch_chained(tile_sums_scan_kernel, dim3(1), dim3(kTsThreads), 0, s, tiles, 0, nullptr,
                        tile_sum, tile_prefix, nullptr, nullptr);
}

cudaError_t launch_tile_counts_scan(int tiles, const int* counts, uint32_t* prefix,
                                    int* total_out, cudaStream_t s, const uint32_t* gate) {
  if (tiles <= 0) return cudaSuccess;
  return launch_chained(tile_sums_scan_kernel, dim3(1), dim3(kTsThreads), 0, s, tiles, 0, nullptr,
                        counts, prefix, total_out, gate);
}

}  // namespace octgb
