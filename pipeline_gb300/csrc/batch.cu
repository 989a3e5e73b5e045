// Batched build: many point clouds of uneven size in one launch sequence.
//
// The clouds are concatenated (cloud c holds points [start_c, start_c + n_c));
// every output array keeps that layout, so cloud c's codes, tree arrays,
// edge counts and prefix sums start at start_c and its OctNodes at
// node_start_c. Each cloud is built exactly as a single build of it would be
// (bit-identical), but every stage runs for all clouds in one launch:
//
//   morton    tiles never cross clouds; each CTA walks a contiguous run of
//             tiles and flushes its shared digit histograms per cloud;
//   sort      reduce-then-scan radix passes: per-tile digit histograms, a
//             per-cloud tile-prefix scan, and the pass kernel driven by tile
//             descriptors (cloud-local positions are absolute indices);
//   unique    the single-cloud run-head count, one scan of all tiles' counts
//             (a tile's offset is its entry minus that of its cloud's first
//             tile) and the compaction that also writes each code's delta to
//             the one before it into the cloud's tree tiles, and each cloud's
//             U from its last tile;
//   tree      the single-cloud tree_nodes kernel over the same 4,096-position
//             tiles (tile map: cloud, cloud start, the cloud's tile range),
//             writing the edge counts and their per-tile sums;
//   scan      one scan of the tile sums for all clouds; a tile's prefix is its
//             entry minus that of its cloud's first tile, so no tile waits;
//   octree    the tags are cleared by the prefix-sum tiles; then one CTA per
//             4,096-node tile (emit) and per 256-slot tile (finalize) of a
//             cloud, reusing the single-cloud node and slot functions on
//             per-cloud views.
//
// The host plan (tile descriptors, cloud starts) is uploaded once; every
// size that depends on the data (U_c, M_c) stays on the device, so a batch
// build is a fixed launch sequence that CUDA graphs capture.
#include <stdio.h>

#include <new>
#include <vector>

#include "lsort.cuh"
#include "octree.cuh"
#include "tree.cuh"

namespace octgb {

constexpr int kBatchTile4k = 4096;  // unique / scan tiles (keys or nodes)

// ---------------------------------------------------------------- helpers --
// Cloud of global index g: largest c with start[c] <= g (start[C] = total).
__device__ __forceinline__ int cloud_of(const int* __restrict__ start, int C, int g) {
  int lo = 0, hi = C - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(start + mid) <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

struct BatchDev {
  int C;
  int N;
  const int* start;       // [C+1] point starts
  const int* node_start;  // [C+1] OctNode starts
  const float* mins;      // [C]
  const float* ranges;    // [C]
  const int4* sort_tiles; // [Ts]
  int Ts;
  const int* cloud_tile0; // [C+1] first sort tile of each cloud
  const int4* tiles4k;    // [T4] {first, end, cloud, first tile of cloud}
  int T4;
  const int4* slot_tiles; // [Tn] {first slot, end slot, cloud, 0}: 256 OctNode slots
  int Tn;
};

// ------------------------------------------------------------------ morton --
template <int RB>
__global__ void __launch_bounds__(256)
    batch_morton_kernel(const float4* __restrict__ pts, uint32_t* __restrict__ keys, BatchDev B,
                        uint32_t* __restrict__ ghist, int passes, uint32_t* __restrict__ status) {
  constexpr int BINS = 1 << RB;
  constexpr int PASSES = (30 + RB - 1) / RB;  // the plan's passes over 30-bit codes
  extern __shared__ uint32_t s_hist[];  // [PASSES * BINS] histograms, then the spread table
  uint32_t* lut = s_hist + PASSES * BINS;
  (void)passes;
  const int t0 = (int)((long long)B.Ts * blockIdx.x / gridDim.x);
  const int t1 = (int)((long long)B.Ts * (blockIdx.x + 1) / gridDim.x);
  for (int i = threadIdx.x; i < PASSES * BINS; i += blockDim.x) s_hist[i] = 0;
  fill_spread_lut(lut);
  __syncthreads();
  bool bad = false;
  int cur = t0 < t1 ? B.sort_tiles[t0].z : -1;
  for (int t = t0; t < t1; ++t) {
    const int4 d = B.sort_tiles[t];
    if (d.z != cur) {  // flush the previous cloud's histograms
      __syncthreads();
      uint32_t* g = ghist + (size_t)cur * PASSES * BINS;
      for (int i = threadIdx.x; i < PASSES * BINS; i += blockDim.x) {
        if (s_hist[i]) atomicAdd(&g[i], s_hist[i]);
        s_hist[i] = 0;
      }
      __syncthreads();
      cur = d.z;
    }
    const float mn = B.mins[d.z], rg = B.ranges[d.z];
    const float scale = __fdiv_rn(1024.0f, rg);
    // four loads in flight per thread, then the tile's tail
    constexpr int U = 4;
    int i = d.x + (int)threadIdx.x;
    for (; i + (U - 1) * (int)blockDim.x < d.y; i += U * (int)blockDim.x) {
      float4 p[U];
#pragma unroll
      for (int u = 0; u < U; ++u) p[u] = ld_stream_f4(pts + i + u * blockDim.x);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        bool ok;
        const uint32_t c = morton_code_lut(p[u].x, p[u].y, p[u].z, mn, rg, scale, lut, ok);
        bad |= !ok;
        keys[i + u * blockDim.x] = c;
#pragma unroll
        for (int ps = 0; ps < PASSES; ++ps)
          atomicAdd(&s_hist[ps * BINS + ((c >> (ps * RB)) & (BINS - 1))], 1u);
      }
    }
    for (; i < d.y; i += blockDim.x) {
      const float4 p = ld_stream_f4(pts + i);
      bool ok;
      const uint32_t c = morton_code_lut(p.x, p.y, p.z, mn, rg, scale, lut, ok);
      bad |= !ok;
      keys[i] = c;
#pragma unroll
      for (int ps = 0; ps < PASSES; ++ps)
        atomicAdd(&s_hist[ps * BINS + ((c >> (ps * RB)) & (BINS - 1))], 1u);
    }
  }
  __syncthreads();
  if (cur >= 0) {
    uint32_t* g = ghist + (size_t)cur * passes * BINS;
    for (int i = threadIdx.x; i < passes * BINS; i += blockDim.x)
      if (s_hist[i]) atomicAdd(&g[i], s_hist[i]);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) raise_status(status, kStatusRange);
}

// base[c][p][d] = start_c + exclusive prefix of cloud c's pass-p histogram.
template <int RB>
__global__ void __launch_bounds__(1024)
    batch_hist_scan_kernel(const uint32_t* __restrict__ ghist, uint32_t* __restrict__ base,
                           BatchDev B, int passes) {
  constexpr int BINS = 1 << RB;
  constexpr int T = BINS < 1024 ? BINS : 1024;
  constexpr int PER = BINS / T;
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t total;
  const int c = blockIdx.x / passes;
  const uint32_t* h = ghist + (size_t)blockIdx.x * BINS;
  uint32_t* o = base + (size_t)blockIdx.x * BINS;
  // launched with exactly T threads (every thread reaches the block scan)
  uint32_t v[PER];
  uint32_t sum = 0;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    v[j] = h[threadIdx.x * PER + j];
    sum += v[j];
  }
  uint32_t ex = block_exclusive_sum<T>(sum, warp_tot, &total) + (uint32_t)B.start[c];
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    o[threadIdx.x * PER + j] = ex;
    ex += v[j];
  }
}

// In place: th[t][d] = where tile t's keys of digit d start, for the tiles of
// cloud blockIdx.x (blocks: clouds x 32-digit groups; 32 digits x
// kTsGroups tile groups per block).
constexpr int kTsGroups = 8;
__global__ void __launch_bounds__(32 * kTsGroups)
    batch_tile_scan_kernel(uint32_t* __restrict__ th, int bins, const uint32_t* __restrict__ base,
                           int passes, int pass, BatchDev B, const uint32_t* __restrict__ gate) {
  if (gate && *gate == 0) return;
  __shared__ uint32_t part[kTsGroups][33];
  const int c = blockIdx.x;
  const int l = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int d = blockIdx.y * 32 + l;
  const int ta = B.cloud_tile0[c], tb = B.cloud_tile0[c + 1];
  const int nt = tb - ta;
  const int t0 = ta + (int)((long long)nt * g / kTsGroups);
  const int t1 = ta + (int)((long long)nt * (g + 1) / kTsGroups);
  uint32_t sum = 0;
  if (d < bins)
    for (int t = t0; t < t1; ++t) sum += th[(size_t)t * bins + d];
  part[g][l] = sum;
  __syncthreads();
  if (d >= bins) return;
  uint32_t run = base[((size_t)c * passes + pass) * bins + d];
  for (int k = 0; k < g; ++k) run += part[k][l];
  for (int t = t0; t < t1; ++t) {
    const uint32_t v = th[(size_t)t * bins + d];
    th[(size_t)t * bins + d] = run;
    run += v;
  }
}

// --------------------------------------------------------- tile schedule --
// A batched kernel's tiles: one per CTA by block index (queue == nullptr), or
// taken from an atomic work queue (zeroed before the build) by persistent
// CTAs, one at a time, until they run out. The CTA calls this between tiles.
__device__ __forceinline__ int next_tile(uint32_t* queue, int& round, int* s_tile) {
  if (!queue) return round++ == 0 ? (int)blockIdx.x : 0x7fffffff;
  __syncthreads();  // the previous tile is done with *s_tile
  if (threadIdx.x == 0) *s_tile = (int)atomicAdd(queue, 1u);
  __syncthreads();
  return *s_tile;
}

// ------------------------------------------------------------ prefix sum --
// Inclusive prefix sum of each cloud's edge counts (written by the tree
// kernels with their per-tile sums, scanned into tile_prefix), and each
// cloud's largest octree slot.
__global__ void __launch_bounds__(256)
    batch_prefix_sum_kernel(BatchDev B, const int* __restrict__ unique_c,
                            const int* __restrict__ ec, int* __restrict__ ps_out,
                            int* __restrict__ max_slot_c, const uint32_t* __restrict__ tile_prefix,
                            OctTags tags, uint32_t* __restrict__ queue) {
  __shared__ int s_tile;
  int round = 0;
  for (int t = next_tile(queue, round, &s_tile); t < B.T4; t = next_tile(queue, round, &s_tile)) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  __shared__ int s_max[8];
  __shared__ int s_hi;
  constexpr int ITEMS = 16;
  // the tile's counts, then its prefix sums, staged so that global accesses
  // are coalesced and each thread still scans 16 consecutive entries (padded:
  // entry j at j + j / 32, conflict-free both ways)
  __shared__ int s_v[256 * ITEMS + 256 * ITEMS / 32];
  const int tid = threadIdx.x;
  const int4 d = B.tiles4k[t];
  const int c = d.z, cs = B.start[c];
  const int n = max(unique_c[c] - 1, 0);  // radix nodes of this cloud
  const int lo = d.x - cs;                // first node of the tile (cloud-local)
  if (lo >= n) continue;
  const int valid = min(256 * ITEMS, n - lo);
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int j = k * 256 + tid;
    s_v[j + (j >> 5)] = j < valid ? ec[cs + lo + j] : 0;
  }
  __syncthreads();
  const int j0 = lo + tid * ITEMS;
  int v[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int j = tid * ITEMS + k;
    v[k] = s_v[j + (j >> 5)];
  }
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) sum += (uint32_t)v[k];
  const uint32_t off = block_exclusive_sum<256>(sum, s_warp, &s_total);
  const uint32_t ex = tile_prefix[t] - tile_prefix[d.w];
  uint32_t run = ex + off;
  int mx = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int i = j0 + k;
    run += (uint32_t)v[k];
    const int j = tid * ITEMS + k;
    s_v[j + (j >> 5)] = (int)run;  // each thread rewrites only its own entries
    if (i < n) {
      const int last = v[k] > 0 ? (int)run + v[k] - 1 : (int)run;
      if (i > 0 && v[k] > 0 && last > mx) mx = last;
      if (i == n - 1 && (int)run > mx) mx = (int)run;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int j = k * 256 + tid;
    if (j < valid) ps_out[cs + lo + j] = s_v[j + (j >> 5)];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((tid & 31) == 0) s_max[tid >> 5] = mx;
  __syncthreads();
  if (tid == 0) {
    int m = 0;
    for (int w = 0; w < 8; ++w) m = max(m, s_max[w]);
    atomicMax(&max_slot_c[c], m);
    s_hi = max(m, (int)(ex + s_total));
  }
  // Clear the cloud's octree tags of the tile's slots: from the tile's
  // exclusive prefix to its largest slot or last prefix (consecutive tiles'
  // intervals meet, so [0, M_c) is cleared before stages 7-8 run).
  __syncthreads();
  const int ns = B.node_start[c];
  const int hi = min(s_hi, B.node_start[c + 1] - ns - 1);
  if (hi >= (int)ex) clear_tag_range(tags, (size_t)ns + ex, (size_t)ns + hi, tid, 256);
  }
}

// ------------------------------------------------------------------ octree --
struct BatchOctDev {
  oct_node* nodes;
  const int* offsets;
  const int* counts;
  const uint32_t* codes;
  const uint8_t* prefix_n;
  const uint8_t* hll;
  const uint8_t* hlr;
  const int* parent;
  const int* left_child;
  const int* unique_c;
  const int* max_slot_c;
  OctTags tags;  // over the whole node capacity
};

struct CloudSizes {
  int c, n_brt, n_oct, cap, ns;
  bool fits;
};

__device__ __forceinline__ CloudSizes cloud_sizes(const BatchDev& B, const BatchOctDev& O, int c) {
  CloudSizes z;
  z.c = c;
  z.n_brt = max(O.unique_c[c] - 1, 0);
  z.n_oct = z.n_brt >= 1 ? O.max_slot_c[c] + 1 : 0;
  z.ns = B.node_start[c];
  z.cap = B.node_start[c + 1] - z.ns;
  z.fits = z.n_oct <= z.cap;
  return z;
}

__device__ __forceinline__ OctArgs cloud_view(const BatchDev& B, const BatchOctDev& O,
                                              const CloudSizes& z) {
  const int cs = B.start[z.c];
  OctArgs a{};
  a.nodes = O.nodes + z.ns;
  a.cap = z.cap;
  a.offsets = O.offsets + cs;
  a.counts = O.counts + cs;
  a.codes = O.codes + cs;
  a.prefix_n = O.prefix_n + cs;
  a.hll = O.hll + cs;
  a.hlr = O.hlr + cs;
  a.parent = O.parent + cs;
  a.left_child = O.left_child + cs;
  a.min_coord = B.mins[z.c];
  a.range = B.ranges[z.c];
  a.n_brt_host = z.n_brt;
  a.n_oct_host = z.n_oct;
  return a;
}

__device__ __forceinline__ OctTags cloud_tags(const BatchOctDev& O, const CloudSizes& z) {
  OctTags t;
  t.child = O.tags.child + (size_t)z.ns * 8;
  t.owner = O.tags.owner + z.ns;
  t.mask = O.tags.mask + z.ns;
  t.cap = z.cap;
  return t;
}

// One CTA per 4,096-node tile of a cloud.
__global__ void __launch_bounds__(256, 6)
    batch_oct_emit_kernel(BatchDev B, BatchOctDev O, uint32_t* __restrict__ status,
                          uint32_t* __restrict__ queue) {
  __shared__ int s_tile;
  int round = 0;
  for (int k = next_tile(queue, round, &s_tile); k < B.T4; k = next_tile(queue, round, &s_tile)) {
    const int4 d = B.tiles4k[k];
    const int c = d.z;
    const CloudSizes z = cloud_sizes(B, O, c);
    if (!z.fits) {
      if (k == d.w && threadIdx.x == 0) raise_status(status, kStatusCapacity);
      continue;
    }
    const int cs = B.start[c];
    const int end = min(d.y - cs, z.n_brt);
    const OctArgs a = cloud_view(B, O, z);
    const OctTags t = cloud_tags(O, z);
    Sizes zz;
    zz.n_brt = z.n_brt;
    zz.n_oct = z.n_oct;
    zz.fits = true;
    for (int i = d.x - cs + (int)threadIdx.x; i < end; i += 256)
      emit_node(kOctMake | kOctLink, i, a, t, zz, status);
  }
}

// One CTA per 256 OctNode slots of a cloud.
__global__ void __launch_bounds__(kFinThreads, 6)
    batch_oct_finalize_kernel(BatchDev B, BatchOctDev O, uint32_t* __restrict__ queue) {
  __shared__ __align__(16) int s_nodes[kFinThreads * kNodeWords];
  __shared__ int s_tile;
  int round = 0;
  for (int k = next_tile(queue, round, &s_tile); k < B.Tn; k = next_tile(queue, round, &s_tile)) {
    const int4 d = B.slot_tiles[k];
    const CloudSizes z = cloud_sizes(B, O, d.z);
    const int p0 = d.x - z.ns;
    const int count = min(d.y - d.x, z.n_oct - p0);
    if (!z.fits || z.n_brt < 1 || count <= 0) continue;
    const OctArgs a = cloud_view(B, O, z);
    const int p = p0 + (int)threadIdx.x;
    if ((int)threadIdx.x < count)
      finalize_slot(true, p, a, cloud_tags(O, z), a.prefix_n[0] / 3,
                    s_nodes + threadIdx.x * kNodeWords);
    bulk_fence_writes();
    __syncthreads();
    int* dst = reinterpret_cast<int*>(O.nodes + d.x);
    const int words = count * kNodeWords;
    if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0 && (words & 3) == 0) {
      // one bulk copy of the staged block (the TMA engine writes it); done
      // before the stage is reused
      if (threadIdx.x == 0) {
        bulk_store_s2g(dst, s_nodes, (uint32_t)words * 4u);
        bulk_wait_all();
      }
      continue;
    }
    int k0 = 0;
    if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
      const int quads = words >> 2;
      const uint4* src4 = reinterpret_cast<const uint4*>(s_nodes);
      uint4* dst4 = reinterpret_cast<uint4*>(dst);
      for (int q = threadIdx.x; q < quads; q += kFinThreads) dst4[q] = src4[q];
      k0 = quads << 2;
    }
    for (int q = k0 + threadIdx.x; q < words; q += kFinThreads) dst[q] = s_nodes[q];
  }
}

__global__ void batch_publish_kernel(BatchDev B, BatchOctDev O, const uint32_t* status,
                                     int* __restrict__ counts) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < B.C; c += gridDim.x * blockDim.x) {
    const CloudSizes z = cloud_sizes(B, O, c);
    counts[4 * c + 0] = O.unique_c[c];
    counts[4 * c + 1] = z.n_brt;
    counts[4 * c + 2] = z.n_oct;
    counts[4 * c + 3] = (int)((z.fits ? 0u : kStatusCapacity) | (*status & ~kStatusCapacity));
  }
}

}  // namespace octgb

// ----------------------------------------------------------------- plan + ABI --
struct oct_batch_plan {
  int C = 0;
  int N = 0;
  int total_cap = 0;
  octgb::SortPlan sp{};
  std::vector<int> start, node_start, cloud_tile0;
  std::vector<int4> sort_tiles, tiles4k, slot_tiles;
  // device tables (caller buffer) offsets
  size_t t_start = 0, t_node_start = 0, t_tile0 = 0, t_sort = 0, t_4k = 0, t_slots = 0,
         tables_bytes = 0;
  // workspace offsets
  size_t w_status = 0, w_queue = 0, w_unique = 0, w_maxslot = 0, w_hist = 0,
         zero_bytes = 0, w_tree = 0, w_base = 0, w_th = 0, w_keys_a = 0, w_keys_b = 0,
         w_tags = 0, ws_bytes = 0;
};

namespace {

using octgb::align_up;

// Batched octree-stage kernels run one CTA per tile (the default: their
// tiles are of equal size, and measured faster) or, when switched on, as
// persistent CTAs taking tiles from an atomic work queue.
bool g_batch_queue = false;

// Grid of a batched tile kernel: one CTA per tile without a queue; with one,
// as many CTAs as fit on the device at once (no more than the tiles).
template <typename K>
int queue_grid(K kernel, int threads, int tiles, const uint32_t* queue) {
  if (!queue) return std::max(tiles, 1);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  return std::max(1, std::min(tiles, per_sm * octgb::device_sm_count()));
}

int batch_fail(cudaError_t e, const char* where) {
  char msg[192];
  snprintf(msg, sizeof(msg), "%s: %s", where, cudaGetErrorString(e));
  octgb::set_last_error(msg);
  return OCT_ERR_CUDA;
}

octgb::BatchDev dev_view(const oct_batch_plan* P, const void* tables, const float* mins,
                         const float* ranges) {
  const char* t = static_cast<const char*>(tables);
  octgb::BatchDev B;
  B.C = P->C;
  B.N = P->N;
  B.start = reinterpret_cast<const int*>(t + P->t_start);
  B.node_start = reinterpret_cast<const int*>(t + P->t_node_start);
  B.mins = mins;
  B.ranges = ranges;
  B.sort_tiles = reinterpret_cast<const int4*>(t + P->t_sort);
  B.Ts = (int)P->sort_tiles.size();
  B.cloud_tile0 = reinterpret_cast<const int*>(t + P->t_tile0);
  B.tiles4k = reinterpret_cast<const int4*>(t + P->t_4k);
  B.T4 = (int)P->tiles4k.size();
  B.slot_tiles = reinterpret_cast<const int4*>(t + P->t_slots);
  B.Tn = (int)P->slot_tiles.size();
  return B;
}

}  // namespace

extern "C" {

OCT_API oct_batch_plan* oct_batch_plan_create(int n_clouds, const int32_t* h_sizes,
                                              const int32_t* h_node_caps) {
  using namespace octgb;
  if (n_clouds < 1 || !h_sizes) return nullptr;
  oct_batch_plan* P = new (std::nothrow) oct_batch_plan();
  if (!P) return nullptr;
  P->C = n_clouds;
  long long N = 0, cap = 0;
  P->start.resize(n_clouds + 1);
  P->node_start.resize(n_clouds + 1);
  for (int c = 0; c < n_clouds; ++c) {
    if (h_sizes[c] < 0 || h_sizes[c] > OCT_MAX_OCTREE_NODES + 1 ||
        (h_node_caps && h_node_caps[c] < 0)) {
      delete P;
      return nullptr;
    }
    P->start[c] = (int)N;
    P->node_start[c] = (int)cap;
    N += h_sizes[c];
    cap += h_node_caps ? h_node_caps[c] : h_sizes[c];
    if (N > OCT_MAX_N || cap > OCT_MAX_N) {
      delete P;
      return nullptr;
    }
  }
  P->start[n_clouds] = (int)N;
  P->node_start[n_clouds] = (int)cap;
  P->N = (int)N;
  P->total_cap = (int)cap;
  SortConfig cfg = get_sort_config();
  cfg.scan = 1;  // batched passes use per-cloud tile prefixes
  P->sp = sort_plan_cfg(P->N, 30, cfg);
  const int tile = P->sp.tile;
  P->cloud_tile0.resize(n_clouds + 1);
  for (int c = 0; c < n_clouds; ++c) {
    P->cloud_tile0[c] = (int)P->sort_tiles.size();
    const int f4 = (int)P->tiles4k.size();
    for (int lo = P->start[c]; lo < P->start[c + 1]; lo += tile)
      P->sort_tiles.push_back(make_int4(lo, std::min(lo + tile, P->start[c + 1]), c, P->cloud_tile0[c]));
    for (int lo = P->start[c]; lo < P->start[c + 1]; lo += kBatchTile4k)
      P->tiles4k.push_back(make_int4(lo, std::min(lo + kBatchTile4k, P->start[c + 1]), c, f4));
    for (int lo = P->node_start[c]; lo < P->node_start[c + 1]; lo += kFinThreads)
      P->slot_tiles.push_back(make_int4(lo, std::min(lo + kFinThreads, P->node_start[c + 1]), c, 0));
  }
  P->cloud_tile0[n_clouds] = (int)P->sort_tiles.size();
  size_t o = 0;
  auto take = [&](size_t b) {
    const size_t at = o;
    o = align_up(o + b, 256);
    return at;
  };
  P->t_start = take(4 * (size_t)(n_clouds + 1));
  P->t_node_start = take(4 * (size_t)(n_clouds + 1));
  P->t_tile0 = take(4 * (size_t)(n_clouds + 1));
  P->t_sort = take(16 * (P->sort_tiles.size() + 1));
  P->t_4k = take(16 * (P->tiles4k.size() + 1));
  P->t_slots = take(16 * (P->slot_tiles.size() + 1));
  P->tables_bytes = o;
  const int passes = P->sp.passes, bins = P->sp.bins;
  o = 0;
  P->w_status = take(4);
  P->w_queue = take(64);  // work-queue counters: prefix sum, emit, finalize
  P->w_unique = take(4 * (size_t)n_clouds);
  P->w_maxslot = take(4 * (size_t)n_clouds);
  P->w_hist = take(4 * (size_t)n_clouds * passes * bins);
  P->zero_bytes = o;
  P->w_tree = take(tree_scratch_bytes_tiles((int)P->tiles4k.size()));
  P->w_base = take(4 * (size_t)n_clouds * passes * bins);
  P->w_th = take(4 * (P->sort_tiles.size() + 1) * bins);
  P->w_keys_a = take(4 * (size_t)std::max(P->N, 1));
  P->w_keys_b = take(4 * (size_t)std::max(P->N, 1));
  P->w_tags = take(oct_tags_bytes(std::max(P->total_cap, 1)));
  P->ws_bytes = o;
  return P;
}

OCT_API void oct_batch_plan_destroy(oct_batch_plan* P) { delete P; }

OCT_API int oct_batch_plan_info(const oct_batch_plan* P, int64_t out[6]) {
  if (!P || !out) return OCT_ERR_INVALID_ARG;
  out[0] = P->C;
  out[1] = P->N;
  out[2] = P->total_cap;
  out[3] = (int64_t)P->tables_bytes;
  out[4] = (int64_t)P->ws_bytes;
  out[5] = (int64_t)P->sort_tiles.size();
  return OCT_OK;
}

OCT_API int oct_batch_upload_tables(const oct_batch_plan* P, void* d_tables, oct_stream_t stream) {
  if (!P || !d_tables || (reinterpret_cast<uintptr_t>(d_tables) & 255)) return OCT_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char* t = static_cast<char*>(d_tables);
  cudaError_t e = cudaMemcpyAsync(t + P->t_start, P->start.data(), 4 * P->start.size(),
                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(t + P->t_node_start, P->node_start.data(), 4 * P->node_start.size(),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(t + P->t_tile0, P->cloud_tile0.data(), 4 * P->cloud_tile0.size(),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !P->sort_tiles.empty())
    e = cudaMemcpyAsync(t + P->t_sort, P->sort_tiles.data(), 16 * P->sort_tiles.size(),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !P->tiles4k.empty())
    e = cudaMemcpyAsync(t + P->t_4k, P->tiles4k.data(), 16 * P->tiles4k.size(),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !P->slot_tiles.empty())
    e = cudaMemcpyAsync(t + P->t_slots, P->slot_tiles.data(), 16 * P->slot_tiles.size(),
                        cudaMemcpyHostToDevice, s);
  // the host vectors live in the plan: wait so the copies have read them
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? OCT_OK : batch_fail(e, "oct_batch_upload_tables");
}

}  // extern "C"

namespace {

// The learned stage-2 sort of a batched build (nullptr: the LSD passes).
struct BatchLearned {
  const char* model;
  octgb::LcdfLayout L;
  int nb;
  char* ws;            // lbatch_flag_bytes() zeroed per build, then the scratch
  uint32_t* d_stats;   // optional: LsortStats (12 words)
};

size_t lbatch_flag_bytes() { return 256; }

int batch_build(const oct_batch_plan* P, const void* d_tables, const oct_vec4* points,
                const float* d_mins, const float* d_ranges, const oct_build_outputs* out,
                int32_t* d_cloud_counts, void* workspace, size_t workspace_bytes,
                oct_stream_t stream, const BatchLearned* lb) {
  using namespace octgb;
  if (!P || !d_tables || !d_mins || !d_ranges || !out || !d_cloud_counts || !workspace ||
      (reinterpret_cast<uintptr_t>(workspace) & 255))
    return OCT_ERR_INVALID_ARG;
  if (workspace_bytes < P->ws_bytes) return OCT_ERR_WORKSPACE;
  if (P->N > 0 && (!points || (reinterpret_cast<uintptr_t>(points) & 15) || !out->codes ||
                   !out->tree.prefix_n || !out->tree.has_leaf_left || !out->tree.has_leaf_right ||
                   !out->tree.left_child || !out->tree.parent || !out->edge_count ||
                   !out->prefix_sum || !out->nodes || out->nodes_capacity < P->total_cap))
    return OCT_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char* w = static_cast<char*>(workspace);
  const BatchDev B = dev_view(P, d_tables, d_mins, d_ranges);
  uint32_t* status = reinterpret_cast<uint32_t*>(w + P->w_status);
  int* unique_c = reinterpret_cast<int*>(w + P->w_unique);
  int* max_slot_c = reinterpret_cast<int*>(w + P->w_maxslot);
  uint32_t* hist = reinterpret_cast<uint32_t*>(w + P->w_hist);
  uint32_t* base = reinterpret_cast<uint32_t*>(w + P->w_base);
  uint32_t* th = reinterpret_cast<uint32_t*>(w + P->w_th);
  uint32_t* ka = reinterpret_cast<uint32_t*>(w + P->w_keys_a);
  uint32_t* kb = reinterpret_cast<uint32_t*>(w + P->w_keys_b);
  const SortPlan& sp = P->sp;
  const int passes = sp.passes, bins = sp.bins, rb = sp.radix_bits;
  const int sms = device_sm_count();
  cudaError_t e = cudaMemsetAsync(w, 0, P->zero_bytes, s);
  if (e != cudaSuccess) return batch_fail(e, "batch: clear");
  uint32_t* fallback = nullptr;  // gate of the LSD passes: LsortStats::fallback
  if (lb) {
    e = cudaMemsetAsync(lb->ws, 0, lbatch_flag_bytes(), s);
    if (e != cudaSuccess) return batch_fail(e, "batch: clear learned flags");
    fallback = &reinterpret_cast<LsortStats*>(lb->ws)->fallback;
  }
  if (P->N > 0) {
    const int mgrid = std::max(1, std::min(B.Ts, sms * 16));
    const size_t msm = 4 * ((size_t)passes * bins + 1024);  // histograms + spread table
    if (passes != (30 + rb - 1) / rb) return OCT_ERR_INVALID_ARG;
    if (rb == 10) {
      batch_morton_kernel<10><<<mgrid, 256, msm, s>>>(reinterpret_cast<const float4*>(points), ka,
                                                      B, hist, passes, status);
      batch_hist_scan_kernel<10><<<P->C * passes, 1024, 0, s>>>(hist, base, B, passes);
    } else {
      batch_morton_kernel<8><<<mgrid, 256, msm, s>>>(reinterpret_cast<const float4*>(points), ka,
                                                     B, hist, passes, status);
      batch_hist_scan_kernel<8><<<P->C * passes, 256, 0, s>>>(hist, base, B, passes);
    }
    // the sorted keys land in the buffer the LSD passes end in
    uint32_t* sorted = (passes & 1) ? kb : ka;
    if (lb) {
      LbatchArgs la{};
      la.keys = ka;
      la.out = sorted;
      la.tiles = B.sort_tiles;
      la.n_tiles = B.Ts;
      la.start = B.start;
      la.cloud_tile0 = B.cloud_tile0;
      la.C = P->C;
      la.n = P->N;
      la.blob = lb->model;
      la.L = lb->L;
      la.nb = lb->nb;
      la.scratch = lb->ws + lbatch_flag_bytes();
      la.stats = reinterpret_cast<LsortStats*>(lb->ws);
      e = launch_lbatch_sort(la, s);
      if (e != cudaSuccess) return batch_fail(e, "batch: learned sort");
      // The learned result must not land in the passes' input (ka): with an
      // even pass count `sorted` is ka, so the learned path is offered for
      // odd pass counts only (host check).
    }
    uint32_t* a = ka;
    uint32_t* b = kb;
    for (int p = 0; p < passes && e == cudaSuccess; ++p) {
      const int shift = p * rb;
      e = launch_tile_hist(rb, a, P->N, shift, B.sort_tiles, B.Ts, th, s, fallback);
      if (e != cudaSuccess) break;
      batch_tile_scan_kernel<<<dim3(P->C, (bins + 31) / 32), 32 * kTsGroups, 0, s>>>(
          th, bins, base, passes, p, B, fallback);
      e = launch_pass(sp, p > 0, a, b, shift, nullptr, nullptr, nullptr, th, status, fallback, s,
                      B.sort_tiles, B.Ts);
      uint32_t* t = a;
      a = b;
      b = t;
    }
    if (e != cudaSuccess) return batch_fail(e, "batch: sort");
    a = sorted;
    void* tree_ws = w + P->w_tree;
    const TreeScratch TS = tree_scratch_carve_tiles(tree_ws, B.T4);
    e = launch_batch_unique_deltas(a, B.tiles4k, B.T4, B.start, out->codes, unique_c, tree_ws, s);
    if (e == cudaSuccess)
      e = launch_batch_radix_tree_from_deltas(B.tiles4k, B.T4, B.start, unique_c, out->codes,
                                              out->tree.prefix_n, out->tree.has_leaf_left,
                                              out->tree.has_leaf_right, out->tree.left_child,
                                              out->tree.parent, out->edge_count, tree_ws, s);
    if (e == cudaSuccess) e = launch_tile_sums_scan(B.T4, TS.tile_sum, TS.tile_prefix, s);
    if (e != cudaSuccess) return batch_fail(e, "batch: tree");
    const OctTags tags = oct_tags_carve(w + P->w_tags, std::max(P->total_cap, 1));
    uint32_t* queue = g_batch_queue ? reinterpret_cast<uint32_t*>(w + P->w_queue) : nullptr;
    batch_prefix_sum_kernel<<<queue_grid(batch_prefix_sum_kernel, 256, B.T4, queue), 256, 0, s>>>(
        B, unique_c, out->edge_count, out->prefix_sum, max_slot_c, TS.tile_prefix, tags, queue);
    BatchOctDev O;
    O.nodes = out->nodes;
    O.offsets = out->prefix_sum;
    O.counts = out->edge_count;
    O.codes = out->codes;
    O.prefix_n = out->tree.prefix_n;
    O.hll = out->tree.has_leaf_left;
    O.hlr = out->tree.has_leaf_right;
    O.parent = out->tree.parent;
    O.left_child = out->tree.left_child;
    O.unique_c = unique_c;
    O.max_slot_c = max_slot_c;
    O.tags = tags;
    batch_oct_emit_kernel<<<queue_grid(batch_oct_emit_kernel, 256, B.T4, queue), 256, 0, s>>>(
        B, O, status, queue ? queue + 4 : nullptr);
    if (B.Tn > 0)
      batch_oct_finalize_kernel<<<queue_grid(batch_oct_finalize_kernel, kFinThreads, B.Tn, queue),
                                  kFinThreads, 0, s>>>(B, O, queue ? queue + 8 : nullptr);
    batch_publish_kernel<<<(P->C + 255) / 256, 256, 0, s>>>(B, O, status, d_cloud_counts);
  } else {
    e = cudaMemsetAsync(d_cloud_counts, 0, 16 * (size_t)P->C, s);
  }
  if (e == cudaSuccess && lb && lb->d_stats)
    e = cudaMemcpyAsync(lb->d_stats, lb->ws, sizeof(LsortStats), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? OCT_OK : batch_fail(e, "oct_build_octree_batch");
}

}  // namespace

extern "C" {

OCT_API int oct_build_octree_batch(const oct_batch_plan* P, const void* d_tables,
                                   const oct_vec4* points, const float* d_mins,
                                   const float* d_ranges, const oct_build_outputs* out,
                                   int32_t* d_cloud_counts, void* workspace,
                                   size_t workspace_bytes, oct_stream_t stream) {
  return batch_build(P, d_tables, points, d_mins, d_ranges, out, d_cloud_counts, workspace,
                     workspace_bytes, stream, nullptr);
}

OCT_API int oct_set_batch_work_queue(int on) {
  if (on != 0 && on != 1) return OCT_ERR_INVALID_ARG;
  g_batch_queue = on == 1;
  return OCT_OK;
}

OCT_API size_t oct_batch_learned_workspace_bytes(const oct_batch_plan* P, int n_buckets) {
  if (!P || n_buckets < 1 || n_buckets > 65536) return 0;
  return octgb::align_up(P->ws_bytes, 256) + lbatch_flag_bytes() +
         octgb::lbatch_scratch_bytes((int)P->sort_tiles.size(), P->C, n_buckets, P->N);
}

OCT_API int oct_build_octree_batch_learned(const oct_batch_plan* P, const void* d_tables,
                                           const oct_vec4* points, const float* d_mins,
                                           const float* d_ranges, const void* model,
                                           int max_segments, int n_buckets,
                                           const oct_build_outputs* out, int32_t* d_cloud_counts,
                                           uint32_t* d_stats, void* workspace,
                                           size_t workspace_bytes, oct_stream_t stream) {
  using namespace octgb;
  if (!P || !model || max_segments < 1 || max_segments > kLcdfMaxSegments || n_buckets < 1 ||
      n_buckets > 65536 || lsort_hist_smem(n_buckets, max_segments) > (size_t)kLsortMaxSmem)
    return OCT_ERR_INVALID_ARG;
  if ((P->sp.passes & 1) == 0) return OCT_ERR_INVALID_ARG;  // see batch_build
  if (!workspace || workspace_bytes < oct_batch_learned_workspace_bytes(P, n_buckets))
    return workspace ? OCT_ERR_WORKSPACE : OCT_ERR_INVALID_ARG;
  BatchLearned lb;
  lb.model = static_cast<const char*>(model);
  lb.L = lcdf_layout(max_segments);
  lb.nb = n_buckets;
  lb.ws = static_cast<char*>(workspace) + align_up(P->ws_bytes, 256);
  lb.d_stats = d_stats;
  return batch_build(P, d_tables, points, d_mins, d_ranges, out, d_cloud_counts, workspace,
                     workspace_bytes, stream, &lb);
}

}  // extern "C"
