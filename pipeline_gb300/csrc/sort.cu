// Stage 1 (Morton encode) and stage 2 (keys-only LSD radix sort) for sm_103a.
//
// Replaces k_ComputeMortonCode (reference include/kernels/01_morton.hpp:9-13,
// kernels/01_morton.cpp:5-14) and k_SimpleRadixSort
// (include/kernels/02_sort.hpp:6-7, kernels/02_sort.cpp:13-118; GPU form
// kernels/cuda/02_sort.cu:208-338, 566-792).
//
// Design: the Morton kernel reads the points once with 128-bit streaming loads
// and, in the same pass, builds the digit histograms of every sort pass in
// shared memory (so the sort needs no separate histogram read). The sort is a
// single-pass-per-digit "OneSweep" LSD radix sort: each tile ranks its keys
// with warp multi-split (match.any), publishes its per-digit counts, resolves
// its global digit offsets by decoupled look-back over earlier tiles, stages
// the keys in shared memory in digit order and scatters them in runs.
// 30-bit Morton keys take 3 passes of 10-bit digits (28 B/key of HBM traffic
// including the histogram read) instead of the reference's 4 passes of 8.
#include <atomic>
#include <cstdlib>
#include <mutex>
#include <tuple>
#include <vector>

#include "kernels.cuh"

namespace octgb {

// --------------------------------------------------------------------------
// Morton encode, optionally fused with the per-pass digit histograms.
// --------------------------------------------------------------------------
template <int RB, bool HIST>
__global__ void __launch_bounds__(256)
    morton_kernel(const float4* __restrict__ pts, uint32_t* __restrict__ keys, long long n,
                  float min_coord, float range, uint32_t* __restrict__ ghist, int passes,
                  uint32_t* __restrict__ status) {
  chain_enter();
  constexpr int BINS = 1 << RB;
  constexpr int PASSES = (30 + RB - 1) / RB;  // the plan's passes over 30-bit codes
  extern __shared__ uint32_t s_hist[];  // [PASSES * BINS] histograms, then the spread table
  uint32_t* lut = s_hist + (HIST ? PASSES * BINS : 0);
  if (HIST)
    for (int i = threadIdx.x; i < PASSES * BINS; i += blockDim.x) s_hist[i] = 0;
  fill_spread_lut(lut);
  __syncthreads();
  (void)passes;
  const float scale = __fdiv_rn(1024.0f, range);
  bool bad = false;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int U = 4;
  for (; i + (U - 1) * stride < n; i += U * stride) {
    float4 p[U];
#pragma unroll
    for (int u = 0; u < U; ++u) p[u] = ld_stream_f4(pts + i + u * stride);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      bool ok;
      const uint32_t c = morton_code_lut(p[u].x, p[u].y, p[u].z, min_coord, range, scale, lut, ok);
      bad |= !ok;
      keys[i + u * stride] = c;
      if (HIST) {
#pragma unroll
        for (int ps = 0; ps < PASSES; ++ps)
          atomicAdd(&s_hist[ps * BINS + ((c >> (ps * RB)) & (BINS - 1))], 1u);
      }
    }
  }
  for (; i < n; i += stride) {
    const float4 p = ld_stream_f4(pts + i);
    bool ok;
    const uint32_t c = morton_code_lut(p.x, p.y, p.z, min_coord, range, scale, lut, ok);
    bad |= !ok;
    keys[i] = c;
    if (HIST) {
#pragma unroll
      for (int ps = 0; ps < PASSES; ++ps)
        atomicAdd(&s_hist[ps * BINS + ((c >> (ps * RB)) & (BINS - 1))], 1u);
    }
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) raise_status(status, kStatusRange);
  if (HIST) {
    for (int b = threadIdx.x; b < PASSES * BINS; b += blockDim.x)
      if (s_hist[b]) atomicAdd(&ghist[b], s_hist[b]);
  }
}

// --------------------------------------------------------------------------
// Digit histograms of existing keys (sort entry point without Morton).
// --------------------------------------------------------------------------
template <int RB>
__global__ void __launch_bounds__(256)
    histogram_kernel(const uint32_t* __restrict__ keys, int n, uint32_t* __restrict__ ghist,
                     int passes, const uint32_t* __restrict__ gate) {
  chain_enter();
  if (gate && *gate == 0) return;
  constexpr int BINS = 1 << RB;
  extern __shared__ uint32_t s_hist[];
  for (int i = threadIdx.x; i < passes * BINS; i += blockDim.x) s_hist[i] = 0;
  __syncthreads();
  const int n4 = (reinterpret_cast<uintptr_t>(keys) & 15u) ? 0 : n >> 2;
  const uint4* k4 = reinterpret_cast<const uint4*>(keys);
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
    const uint4 v = __ldcs(k4 + i);
    const uint32_t c[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int u = 0; u < 4; ++u)
      for (int ps = 0; ps < passes; ++ps)
        atomicAdd(&s_hist[ps * BINS + ((c[u] >> (ps * RB)) & (BINS - 1))], 1u);
  }
  for (int i = (n4 << 2) + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t c = keys[i];
    for (int ps = 0; ps < passes; ++ps)
      atomicAdd(&s_hist[ps * BINS + ((c >> (ps * RB)) & (BINS - 1))], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < passes * BINS; b += blockDim.x)
    if (s_hist[b]) atomicAdd(&ghist[b], s_hist[b]);
}

// Exclusive scan of each pass's histogram: one block of BINS/… threads per pass.
template <int RB>
__global__ void __launch_bounds__(1024) hist_scan_kernel(const uint32_t* __restrict__ ghist,
                                                         uint32_t* __restrict__ base,
                                                         const uint32_t* __restrict__ gate) {
  chain_enter();
  if (gate && *gate == 0) return;
  constexpr int BINS = 1 << RB;
  constexpr int T = BINS < 1024 ? BINS : 1024;
  constexpr int PER = BINS / T;
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t total;
  const uint32_t* h = ghist + blockIdx.x * BINS;
  uint32_t* o = base + blockIdx.x * BINS;
  uint32_t v[PER];
  uint32_t sum = 0;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    v[j] = h[threadIdx.x * PER + j];
    sum += v[j];
  }
  uint32_t ex = block_exclusive_sum<T>(sum, warp_tot, &total);
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    o[threadIdx.x * PER + j] = ex;
    ex += v[j];
  }
}

// --------------------------------------------------------------------------
// One LSD digit pass over tiles of WARPS*32*ITEMS keys.
//
// Ranking (position of a key among the tile's keys with its digit):
//   STABLE  warp multi-split from RB ballots (peers = lanes with the same
//           digit), counted per warp in shared memory, then offset across
//           warps: stable in (warp, item, lane) order, which is input order.
//   !STABLE one shared-memory atomicAdd per key: any order. Only the first
//           LSD pass may use it (its input order carries no information).
// Tile offsets (where the tile's keys of each digit start in the output):
//   SCAN 0  decoupled look-back over earlier tiles (OneSweep): a tile takes
//           the next id from an atomic counter, publishes its per-digit
//           counts, sums earlier tiles' counts back to an inclusive prefix
//           (bounded waits, windowed relaxed loads).
//   SCAN 1  precomputed: a per-tile digit histogram kernel and a tile-prefix
//           scan ran before the pass (reduce-then-scan); no inter-tile waits.
//   lookback[tile * BINS + b]: bits 31..30 flag (0 not ready, 1 tile count,
//   2 inclusive count of tiles 0..tile), bits 29..0 the count.
// --------------------------------------------------------------------------
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1;

__device__ __forceinline__ void st_relaxed_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Decoupled look-back for digit b of tile `tile` (> 0) over the per-tile words
// lookback[t * BINS + b] (flag in the top two bits, count below): first probe
// the immediate predecessor, then windows of kWin predecessor words (relaxed
// loads, all in flight), summing aggregates until an inclusive word. Publishes
// the tile's inclusive value and returns its exclusive prefix. A word that is
// not published within limit_ns makes the wait give up (status bit set; the
// prefix is then meaningless and the caller's scatter stays in bounds).
template <int BINS>
__device__ __forceinline__ uint32_t digit_lookback(uint32_t* lookback, int tile, int b,
                                                  uint32_t own, uint32_t* status,
                                                  unsigned long long limit_ns) {
  constexpr int kWin = 16;
  uint32_t prefix = 0;
  int pred = tile - 1;
  WaitBound wait(limit_ns);
  bool done = false;
  {
    uint32_t w0 = ld_relaxed_u32(lookback + (size_t)pred * BINS + b);
    while ((w0 & kFlagMask) == 0) {
      if (wait.expired()) {
        raise_status(status, kStatusSpinTimeout);
        done = true;
        break;
      }
      w0 = ld_relaxed_u32(lookback + (size_t)pred * BINS + b);
    }
    prefix += w0 & kValMask;
    done = done || (w0 & kFlagMask) == kFlagInc;
    --pred;
  }
  while (!done) {
    uint32_t w[kWin];
#pragma unroll
    for (int k = 0; k < kWin; ++k)
      w[k] = (pred - k >= 0) ? ld_relaxed_u32(lookback + (size_t)(pred - k) * BINS + b) : kFlagInc;
    bool stop = false;
    int adv = 0;
#pragma unroll
    for (int k = 0; k < kWin; ++k) {
      const uint32_t f = w[k] & kFlagMask;
      if (!stop) {
        if (f == 0) {
          stop = true;
        } else {
          prefix += w[k] & kValMask;
          ++adv;
          if (f == kFlagInc) stop = done = true;
        }
      }
    }
    if (done) break;
    pred -= adv;
    if (adv < kWin && wait.expired()) {  // stopped at a word not ready yet: poll it again
      raise_status(status, kStatusSpinTimeout);
      break;
    }
  }
  st_relaxed_u32(lookback + (size_t)tile * BINS + b, kFlagInc | ((prefix + own) & kValMask));
  return prefix;
}

template <int RB, int WARPS, int ITEMS, bool STABLE>
struct PassSmem {
  static constexpr int BINS = 1 << RB;
  static constexpr int TILE = WARPS * 32 * ITEMS;
  static constexpr int HIST_BYTES = STABLE ? WARPS * BINS * 2 : BINS * 4;
  static constexpr int STAGE_BYTES = TILE * 4;
  // the stable per-warp counters are dead once positions are known: alias them
  static constexpr int UNION_BYTES =
      STABLE ? (HIST_BYTES > STAGE_BYTES ? HIST_BYTES : STAGE_BYTES) : HIST_BYTES + STAGE_BYTES;
  static constexpr int BYTES = UNION_BYTES + BINS * 4 * 2 + 64 * 4;
};

template <int RB, int WARPS, int ITEMS, bool STABLE, int SCAN>
__global__ void __launch_bounds__(WARPS * 32, (ITEMS <= 16 ? 2 : 1))
    sort_pass_kernel(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int n,
                     int shift, const uint32_t* __restrict__ bin_base,
                     uint32_t* __restrict__ lookback, uint32_t* __restrict__ tile_counter,
                     const uint32_t* __restrict__ tile_prefix, uint32_t* __restrict__ status,
                     const uint32_t* __restrict__ gate, const int4* __restrict__ tdesc,
                     DigitAlt alt) {
  chain_enter();
  if (gate && *gate == 0) return;
  // The MSD form's top-digit scatter: the order inside a bucket is free, so a
  // tile takes its digit runs' places with one atomic add per digit on the
  // bucket's cursor (alt.part, 16 words apart) instead of the tile scan.
  bool cursors = false;
  if (alt.flag && *alt.flag) {
    shift = alt.shift;
    bin_base = alt.base;
    cursors = !STABLE && SCAN == 1;
  }
  using L = PassSmem<RB, WARPS, ITEMS, STABLE>;
  constexpr int BINS = L::BINS, THREADS = WARPS * 32, TILE = L::TILE;
  constexpr uint32_t MASK = BINS - 1;
  extern __shared__ __align__(16) unsigned char smem[];
  uint16_t* whist = reinterpret_cast<uint16_t*>(smem);             // STABLE: [WARPS][BINS]
  uint32_t* cnt = reinterpret_cast<uint32_t*>(smem);               // !STABLE: [BINS]
  uint32_t* stage = reinterpret_cast<uint32_t*>(smem + (STABLE ? 0 : L::HIST_BYTES));  // [TILE]
  uint32_t* bin_local = reinterpret_cast<uint32_t*>(smem + L::UNION_BYTES);  // [BINS]
  uint32_t* bin_glob = bin_local + BINS;                                      // [BINS]
  uint32_t* misc = bin_glob + BINS;                                           // [64]

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (SCAN == 0) {
    if (tid == 0) misc[0] = atomicAdd(tile_counter, 1u);
  }
  if (STABLE) {
    for (int i = tid; i < WARPS * BINS / 2; i += THREADS) reinterpret_cast<uint32_t*>(whist)[i] = 0;
  } else {
    for (int i = tid; i < BINS; i += THREADS) cnt[i] = 0;
  }
  __syncthreads();
  const int tile = SCAN == 0 ? (int)misc[0] : (int)blockIdx.x;
  // Batched sorts pass tile descriptors {first key, end key, cloud, first tile
  // of the cloud}: a tile never crosses a cloud boundary.
  const int tile_start = tdesc ? tdesc[tile].x : tile * TILE;
  const int tile_end = tdesc ? tdesc[tile].y : n;
  const int valid = min(TILE, tile_end - tile_start);

  // Load (warp-striped: item-major within each warp's contiguous segment).
  uint32_t key[ITEMS];
  const int wbase = tile_start + warp * 32 * ITEMS;
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    const int idx = wbase + it * 32 + lane;
    key[it] = idx < tile_end ? __ldcs(src + idx) : 0xffffffffu;
  }

  uint16_t rank[ITEMS];
  if (STABLE) {
    uint16_t* wh = whist + warp * BINS;
    const uint32_t lt = lanemask_lt();
    // Peers split the digit into a low and a high half of at most 5 bits:
    // lane v builds the mask of lanes whose low (high) half equals v from the
    // ballots of those bits, and a lane fetches the entries of its own halves.
    constexpr int LOB = RB / 2, HIB = RB - LOB;
    uint32_t lane_bits[HIB];  // all ones where the lane index has bit k
#pragma unroll
    for (int b = 0; b < HIB; ++b) lane_bits[b] = 0u - ((uint32_t)(lane >> b) & 1u);
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
      const uint32_t d = (key[it] >> shift) & MASK;
      uint32_t eq_lo = 0xffffffffu, eq_hi = 0xffffffffu;
#pragma unroll
      for (int b = 0; b < LOB; ++b)
        eq_lo &= ~(__ballot_sync(0xffffffffu, (d >> b) & 1u) ^ lane_bits[b]);
#pragma unroll
      for (int b = 0; b < HIB; ++b)
        eq_hi &= ~(__ballot_sync(0xffffffffu, (d >> (LOB + b)) & 1u) ^ lane_bits[b]);
      const uint32_t peers = __shfl_sync(0xffffffffu, eq_lo, (int)(d & ((1u << LOB) - 1u))) &
                             __shfl_sync(0xffffffffu, eq_hi, (int)(d >> LOB));
      const uint32_t before = wh[d];
      rank[it] = (uint16_t)(before + __popc(peers & lt));
      __syncwarp();
      if ((peers & lt) == 0) wh[d] = (uint16_t)(before + __popc(peers));
      __syncwarp();
    }
  } else {
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
      const int idx = wbase + it * 32 + lane;
      rank[it] = idx < tile_end ? (uint16_t)atomicAdd(&cnt[(key[it] >> shift) & MASK], 1u)
                                : (uint16_t)0;
    }
  }
  __syncthreads();

  // Per-digit tile counts (stable: plus exclusive offsets across warps), publish.
  const int invalid = TILE - valid;
  constexpr int PER_T = (BINS + THREADS - 1) / THREADS;
  uint32_t own[PER_T];
#pragma unroll
  for (int j = 0; j < PER_T; ++j) {
    const int b = tid + j * THREADS;
    if (b >= BINS) break;
    uint32_t run = 0;
    if (STABLE) {
#pragma unroll
      for (int w = 0; w < WARPS; ++w) {
        const uint32_t c = whist[w * BINS + b];
        whist[w * BINS + b] = (uint16_t)run;
        run += c;
      }
      own[j] = run - (b == (int)MASK ? (uint32_t)invalid : 0u);  // padding ranks last
    } else {
      run = cnt[b];  // padding keys took no rank
      own[j] = run;
    }
    bin_local[b] = run;
    if (SCAN == 0)
      st_relaxed_u32(lookback + (size_t)tile * BINS + b, (tile == 0 ? kFlagInc : kFlagAgg) | own[j]);
    if (SCAN == 1 && cursors)
      bin_glob[b] = bin_base[b] + (own[j] ? atomicAdd(alt.part + (size_t)b * kCursorStride, own[j])
                                          : 0u);
  }
  __syncthreads();

  // Exclusive scan of the tile counts over digits -> local digit starts.
  {
    constexpr int PER = (BINS + THREADS - 1) / THREADS;
    uint32_t v[PER];
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int b = tid * PER + j;
      v[j] = b < BINS ? bin_local[b] : 0u;
      s += v[j];
    }
    uint32_t ex = block_exclusive_sum<THREADS>(s, misc + 8, misc + 4);
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int b = tid * PER + j;
      if (b < BINS) bin_local[b] = ex;
      ex += v[j];
    }
  }
  __syncthreads();

  if (SCAN == 1) {
    if (cursors) {
      for (int b = tid; b < BINS; b += THREADS) bin_glob[b] -= bin_local[b];
    } else {
      for (int b = tid; b < BINS; b += THREADS)
        bin_glob[b] = tile_prefix[(size_t)tile * BINS + b] - bin_local[b];
    }
  } else {
    // Decoupled look-back per digit (digit_lookback).
#pragma unroll
    for (int j = 0; j < PER_T; ++j) {
      const int b = tid + j * THREADS;
      if (b >= BINS) break;
      const uint32_t prefix =
          tile > 0 ? digit_lookback<BINS>(lookback, tile, b, own[j], status, kWaitLimitNs) : 0u;
      bin_glob[b] = bin_base[b] + prefix - bin_local[b];
    }
  }

  // Local positions (read before the staging area overwrites the counters).
  uint16_t pos[ITEMS];
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    const uint32_t d = (key[it] >> shift) & MASK;
    pos[it] = (uint16_t)(bin_local[d] + (STABLE ? whist[warp * BINS + d] : 0u) + rank[it]);
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    if (STABLE || wbase + it * 32 + lane < tile_end) stage[pos[it]] = key[it];
  }
  __syncthreads();

  // Scatter in digit runs; padding keys sit at [valid, TILE) and are skipped.
  bool oob = false;
#pragma unroll 4
  for (int j = tid; j < valid; j += THREADS) {
    const uint32_t k = stage[j];
    const uint32_t g = bin_glob[(k >> shift) & MASK] + (uint32_t)j;
    if (g < (uint32_t)n)
      dst[g] = k;
    else
      oob = true;  // only after a look-back timeout: never write out of bounds
  }
  if (oob) raise_status(status, kStatusSpinTimeout);
}

// Per-tile digit counts for SCAN 1 passes: th[tile * BINS + b].
// Reduce-then-scan over tiles: the tiles are cut into kScanSplits contiguous
// splits; tile_hist also adds each tile's counts into its split's partial
// sums, so the tile scan runs every split in its own CTAs.
constexpr int kScanSplits = 16;
// the MSD form's bucket cursors live in the top digit's split sums
static_assert(kCursorStride <= kScanSplits, "one cursor per digit in the split sums");

__host__ __device__ __forceinline__ int split_tiles(int tiles) {
  return (tiles + kScanSplits - 1) / kScanSplits;
}

template <int RB>
__global__ void __launch_bounds__(256)
    tile_hist_kernel(const uint32_t* __restrict__ keys, int n, int shift, int tile_keys,
                     uint32_t* __restrict__ th, const uint32_t* __restrict__ gate,
                     const int4* __restrict__ tdesc, uint32_t* __restrict__ part, int tiles) {
  chain_enter();
  if (gate && *gate == 0) return;
  constexpr int BINS = 1 << RB;
  __shared__ uint32_t h[BINS];
  // CTAs walk the tiles (a capped grid: a gated-off launch schedules few CTAs)
  for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
    for (int b = threadIdx.x; b < BINS; b += 256) h[b] = 0;
    __syncthreads();
    const int lo = tdesc ? tdesc[t].x : t * tile_keys;
    const int hi = tdesc ? tdesc[t].y : min(n, lo + tile_keys);
    const bool vec = ((reinterpret_cast<uintptr_t>(keys + lo)) & 15u) == 0;
    const int n4 = vec ? (hi - lo) >> 2 : 0;
    const uint4* k4 = reinterpret_cast<const uint4*>(keys + lo);
    for (int i = threadIdx.x; i < n4; i += 256) {
      const uint4 v = __ldcs(k4 + i);
      atomicAdd(&h[(v.x >> shift) & (BINS - 1)], 1u);
      atomicAdd(&h[(v.y >> shift) & (BINS - 1)], 1u);
      atomicAdd(&h[(v.z >> shift) & (BINS - 1)], 1u);
      atomicAdd(&h[(v.w >> shift) & (BINS - 1)], 1u);
    }
    for (int i = lo + 4 * n4 + threadIdx.x; i < hi; i += 256)
      atomicAdd(&h[(keys[i] >> shift) & (BINS - 1)], 1u);
    __syncthreads();
    for (int b = threadIdx.x; b < BINS; b += 256) th[(size_t)t * BINS + b] = h[b];
    if (part) {
      uint32_t* ps = part + (size_t)(t / split_tiles(tiles)) * BINS;
      for (int b = threadIdx.x; b < BINS; b += 256)
        if (h[b]) atomicAdd(ps + b, h[b]);
    }
    __syncthreads();  // h is the next tile's
  }
}

// Grid of the tile-histogram kernel of the gated whole-build passes: the
// tiles, capped at 8 CTAs per SM.
static int tile_hist_grid(int tiles) {
  const int cap = device_sm_count() * 8;
  return tiles < cap ? tiles : cap;
}

// In place: th[t][b] becomes the output index where tile t's keys of digit b
// start (bin_base[b] + counts of earlier tiles). Block: 32 digits x 32 tile
// groups of one split (blockIdx.y); lanes run along digits, so every load is a
// coalesced 128 B row part. A split starts from the partial sums of the
// splits before it.
__global__ void __launch_bounds__(1024)
    tile_scan_split_kernel(uint32_t* __restrict__ th, int tiles, int bins,
                           const uint32_t* __restrict__ bin_base, const uint32_t* __restrict__ part,
                           const uint32_t* __restrict__ gate) {
  chain_enter();
  if (gate && *gate == 0) return;
  __shared__ uint32_t sums[32][33];
  const int l = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int d = blockIdx.x * 32 + l;
  const int per = split_tiles(tiles);
  const int ta = blockIdx.y * per, tb = min(tiles, ta + per);
  const int nt = max(tb - ta, 0);
  const int t0 = ta + nt * g / 32, t1 = ta + nt * (g + 1) / 32;
  uint32_t sum = 0;
  if (d < bins)
    for (int t = t0; t < t1; ++t) sum += th[(size_t)t * bins + d];
  sums[g][l] = sum;
  __syncthreads();
  if (d >= bins) return;
  uint32_t run = bin_base[d];
  for (int s = 0; s < (int)blockIdx.y; ++s) run += part[(size_t)s * bins + d];
  for (int k = 0; k < g; ++k) run += sums[k][l];
  for (int t = t0; t < t1; ++t) {
    const uint32_t v = th[(size_t)t * bins + d];
    th[(size_t)t * bins + d] = run;
    run += v;
  }
}

// --------------------------------------------------------------------------
// Host-side planning and launch.
// --------------------------------------------------------------------------
static SortConfig g_default_cfg = {10, 16, 16, 1};

void set_sort_config(const SortConfig& c) { g_default_cfg = c; }
SortConfig get_sort_config() { return g_default_cfg; }

static bool valid_config(const SortConfig& c) {
  return ((c.radix_bits == 10 && c.warps == 16 && (c.items == 16 || c.items == 24)) ||
          (c.radix_bits == 8 && c.warps == 16 && (c.items == 16 || c.items == 24))) &&
         (c.scan == 0 || c.scan == 1);
}

SortPlan sort_plan_cfg(int n, int key_bits, SortConfig cfg) {
  if (!valid_config(cfg)) cfg = SortConfig{10, 16, 16, 1};
  SortPlan p{};
  p.n = n;
  p.cfg = cfg;
  // 30-bit keys: the configured digit width; wider keys: 8-bit digits.
  p.radix_bits = key_bits <= 30 ? cfg.radix_bits : 8;
  if (p.radix_bits == 8 && cfg.radix_bits != 8) p.cfg.items = 16;
  p.cfg.radix_bits = p.radix_bits;
  p.passes = (key_bits + p.radix_bits - 1) / p.radix_bits;
  if (p.passes < 1) p.passes = 1;
  p.bins = 1 << p.radix_bits;
  p.tile = p.cfg.warps * 32 * p.cfg.items;
  p.tiles = n > 0 ? (n + p.tile - 1) / p.tile : 0;
  // zeroed per sort: hist, counters, look-back (scan 0); then base and the
  // per-tile histograms (scan 1), which are fully written before being read.
  p.hist_off = 0;
  p.counter_off = align_up(p.hist_off + sizeof(uint32_t) * p.passes * p.bins, 256);
  p.lookback_off = align_up(p.counter_off + sizeof(uint32_t) * 64, 256);
  const size_t lb_bytes = p.cfg.scan == 0 ? sizeof(uint32_t) * (size_t)p.passes * p.tiles * p.bins : 0;
  p.tile_part_off = align_up(p.lookback_off + lb_bytes, 256);
  const size_t part_bytes =
      p.cfg.scan == 1 ? sizeof(uint32_t) * (size_t)p.passes * kScanSplits * p.bins : 0;
  p.zero_bytes = align_up(p.tile_part_off + part_bytes, 256);
  p.base_off = p.zero_bytes;
  p.tile_hist_off = align_up(p.base_off + sizeof(uint32_t) * p.passes * p.bins, 256);
  const size_t th_bytes = p.cfg.scan == 1 ? sizeof(uint32_t) * (size_t)p.tiles * p.bins : 0;
  p.bytes = align_up(p.tile_hist_off + th_bytes, 256);
  return p;
}

SortPlan sort_plan(int n, int key_bits) { return sort_plan_cfg(n, key_bits, g_default_cfg); }

// Per-device caches: the SM count, and the dynamic shared-memory limits
// already raised (a kernel attribute belongs to one device's context).
namespace {
constexpr int kMaxDevices = 64;
std::atomic<int> g_num_sms[kMaxDevices];
std::mutex g_attr_mu;
std::vector<std::tuple<int, const void*, int>> g_attr_set;

int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
  return dev;
}
}  // namespace

int device_sm_count() {
  const int dev = current_device();
  if (dev >= kMaxDevices) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 152;
  }
  int v = g_num_sms[dev].load(std::memory_order_relaxed);
  if (v == 0) {
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    if (v <= 0) v = 152;
    g_num_sms[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

bool chained_launches() {
  static const bool on = [] {
    const char* v = std::getenv("OCT_PDL");
    return !(v && v[0] == '0' && v[1] == '\0');
  }();
  return on;
}

cudaError_t set_smem_limit(const void* func, int bytes) {
  const int dev = current_device();
  std::lock_guard<std::mutex> lock(g_attr_mu);
  for (const auto& t : g_attr_set)
    if (std::get<0>(t) == dev && std::get<1>(t) == func && std::get<2>(t) >= bytes)
      return cudaSuccess;
  const cudaError_t e =
      cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) g_attr_set.emplace_back(dev, func, bytes);
  return e;
}

// Diagnostics: one digit look-back of tile 1 whose predecessor (tile 0) never
// publishes; it must give up after limit_ns with the status bit set.
__global__ void diag_digit_wait_kernel(uint32_t* lookback, uint32_t* status,
                                       unsigned long long limit_ns) {
  if (threadIdx.x == 0) digit_lookback<1024>(lookback, 1, 0, 1u, status, limit_ns);
}

cudaError_t launch_diag_sort_wait(uint32_t* lookback, uint32_t* status,
                                  unsigned long long limit_ns, cudaStream_t s) {
  diag_digit_wait_kernel<<<1, 32, 0, s>>>(lookback, status, limit_ns);
  return cudaGetLastError();
}

template <int RB, int WARPS, int ITEMS, bool STABLE, int SCAN>
static cudaError_t launch_pass_t(const uint32_t* src, uint32_t* dst, int n, int shift,
                                 const uint32_t* base, uint32_t* lookback, uint32_t* counter,
                                 const uint32_t* tile_prefix, uint32_t* status,
                                 const uint32_t* gate, cudaStream_t s, const int4* tdesc,
                                 int tiles_override, DigitAlt alt) {
  using L = PassSmem<RB, WARPS, ITEMS, STABLE>;
  auto k = sort_pass_kernel<RB, WARPS, ITEMS, STABLE, SCAN>;
  const cudaError_t ea = set_smem_limit(reinterpret_cast<const void*>(k), L::BYTES);
  if (ea != cudaSuccess) return ea;
  const int tiles = tiles_override > 0 ? tiles_override : (n + L::TILE - 1) / L::TILE;
  return launch_chained(k, dim3(tiles), dim3(WARPS * 32), L::BYTES, s, src, dst, n, shift, base,
                        lookback, counter, tile_prefix, status, gate, tdesc, alt);
}

template <int RB, int WARPS, int ITEMS>
static cudaError_t launch_pass_cfg(bool stable, int scan, const uint32_t* src, uint32_t* dst,
                                   int n, int shift, const uint32_t* base, uint32_t* lookback,
                                   uint32_t* counter, const uint32_t* tile_prefix,
                                   uint32_t* status, const uint32_t* gate, cudaStream_t s,
                                   const int4* tdesc, int tiles, DigitAlt alt) {
  if (stable)
    return scan == 0 ? launch_pass_t<RB, WARPS, ITEMS, true, 0>(src, dst, n, shift, base, lookback,
                                                                 counter, tile_prefix, status, gate, s, tdesc, tiles, alt)
                     : launch_pass_t<RB, WARPS, ITEMS, true, 1>(src, dst, n, shift, base, lookback,
                                                                 counter, tile_prefix, status, gate, s, tdesc, tiles, alt);
  return scan == 0 ? launch_pass_t<RB, WARPS, ITEMS, false, 0>(src, dst, n, shift, base, lookback,
                                                                counter, tile_prefix, status, gate, s, tdesc, tiles, alt)
                   : launch_pass_t<RB, WARPS, ITEMS, false, 1>(src, dst, n, shift, base, lookback,
                                                                counter, tile_prefix, status, gate, s, tdesc, tiles, alt);
}

cudaError_t launch_pass(const SortPlan& p, bool stable, const uint32_t* src, uint32_t* dst,
                        int shift, const uint32_t* base, uint32_t* lookback, uint32_t* counter,
                        const uint32_t* tile_prefix, uint32_t* status, const uint32_t* gate,
                        cudaStream_t s, const int4* tdesc, int tiles, DigitAlt alt) {
  const int sc = p.cfg.scan;
  if (p.radix_bits == 10) {
    if (p.cfg.items == 24)
      return launch_pass_cfg<10, 16, 24>(stable, sc, src, dst, p.n, shift, base, lookback, counter,
                                         tile_prefix, status, gate, s, tdesc, tiles, alt);
    return launch_pass_cfg<10, 16, 16>(stable, sc, src, dst, p.n, shift, base, lookback, counter,
                                       tile_prefix, status, gate, s, tdesc, tiles, alt);
  }
  if (p.cfg.items == 24)
    return launch_pass_cfg<8, 16, 24>(stable, sc, src, dst, p.n, shift, base, lookback, counter,
                                      tile_prefix, status, gate, s, tdesc, tiles, alt);
  return launch_pass_cfg<8, 16, 16>(stable, sc, src, dst, p.n, shift, base, lookback, counter,
                                    tile_prefix, status, gate, s, tdesc, tiles, alt);
}

cudaError_t launch_morton(const float4* pts, uint32_t* keys, long long n, float min_coord,
                          float range, const SortPlan* plan, void* ctrl, uint32_t* status,
                          cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int blocks = device_sm_count() * 6;
  long long need = (n + 255) / 256;
  const int grid = (int)(need < blocks ? need : blocks);
  if (plan) {
    if (plan->passes != (30 + plan->radix_bits - 1) / plan->radix_bits) return cudaErrorInvalidValue;
    uint32_t* hist = reinterpret_cast<uint32_t*>(static_cast<char*>(ctrl) + plan->hist_off);
    const size_t sm = sizeof(uint32_t) * (plan->passes * plan->bins + 1024);
    if (plan->radix_bits == 10)
      return launch_chained(morton_kernel<10, true>, dim3(grid), dim3(256), sm, s, pts, keys, n,
                            min_coord, range, hist, plan->passes, status);
    return launch_chained(morton_kernel<8, true>, dim3(grid), dim3(256), sm, s, pts, keys, n,
                          min_coord, range, hist, plan->passes, status);
  }
  return launch_chained(morton_kernel<10, false>, dim3(grid), dim3(256), sizeof(uint32_t) * 1024, s,
                        pts, keys, n, min_coord, range, nullptr, 0, status);
}

cudaError_t launch_histogram_gated(const uint32_t* keys, const SortPlan* plan, void* ctrl,
                                   const uint32_t* gate, cudaStream_t s) {
  if (plan->n <= 0) return cudaSuccess;
  uint32_t* hist = reinterpret_cast<uint32_t*>(static_cast<char*>(ctrl) + plan->hist_off);
  const size_t sm = sizeof(uint32_t) * plan->passes * plan->bins;
  const int blocks = device_sm_count() * 2;
  int need = (plan->n / 4 + 255) / 256 + 1;
  const int grid = need < blocks ? need : blocks;
  if (plan->radix_bits == 10)
    return launch_chained(histogram_kernel<10>, dim3(grid), dim3(256), sm, s, keys, plan->n, hist,
                          plan->passes, gate);
  return launch_chained(histogram_kernel<8>, dim3(grid), dim3(256), sm, s, keys, plan->n, hist,
                        plan->passes, gate);
}

cudaError_t launch_histogram(const uint32_t* keys, const SortPlan* plan, void* ctrl,
                             cudaStream_t s) {
  return launch_histogram_gated(keys, plan, ctrl, nullptr, s);
}

static cudaError_t sort_passes_impl(uint32_t* keys, uint32_t* alt, const SortPlan* plan,
                                    void* ctrl, uint32_t* status, const uint32_t* gate,
                                    cudaStream_t s, uint32_t** result, Recorder* rec,
                                    const uint32_t* msd_flag = nullptr,
                                    const uint32_t* lsd_flag = nullptr) {
  *result = keys;
  if (plan->n <= 1) return cudaSuccess;
  char* c = static_cast<char*>(ctrl);
  uint32_t* hist = reinterpret_cast<uint32_t*>(c + plan->hist_off);
  uint32_t* base = reinterpret_cast<uint32_t*>(c + plan->base_off);
  uint32_t* counters = reinterpret_cast<uint32_t*>(c + plan->counter_off);
  uint32_t* lookback = reinterpret_cast<uint32_t*>(c + plan->lookback_off);
  uint32_t* th = reinterpret_cast<uint32_t*>(c + plan->tile_hist_off);
  uint32_t* part = reinterpret_cast<uint32_t*>(c + plan->tile_part_off);
  cudaError_t e =
      plan->radix_bits == 10
          ? launch_chained(hist_scan_kernel<10>, dim3(plan->passes), dim3(1024), 0, s, hist, base,
                           gate) : launch_chained(hist_scan_kernel<8>, dim3(plan->passes),
                           dim3(256), 0, s, hist, base, gate);
  if (e != cudaSuccess) return e;
  mark(rec, s);
  // The MSD form's top-digit scatter reuses pass 0's pass launch (unstable,
  // the top digit's shift and bases, its places from bucket cursors kept in
  // the top digit's zeroed split sums, chosen on the device); the later passes
  // then return at once.
  DigitAlt alt0;
  if (msd_flag && msd_plan_ok(*plan)) {
    const int top = plan->passes - 1;
    alt0.flag = msd_flag;
    alt0.shift = top * plan->radix_bits;
    alt0.base = base + (size_t)top * plan->bins;
    alt0.part = part + (size_t)top * kScanSplits * plan->bins;
  }
  uint32_t* a = keys;
  uint32_t* b = alt;
  for (int p = 0; p < plan->passes; ++p) {
    const int shift = p * plan->radix_bits;
    const uint32_t* g = (p > 0 && lsd_flag) ? lsd_flag : gate;
    const DigitAlt da = p == 0 ? alt0 : DigitAlt{};
    if (plan->cfg.scan == 1) {
      // the MSD form's scatter takes its places from the bucket cursors: the
      // tile histograms and their scan run for the LSD form only
      const uint32_t* gs = (p == 0 && alt0.flag) ? lsd_flag : g;
      uint32_t* pp = part + (size_t)p * kScanSplits * plan->bins;
      const dim3 hg(tile_hist_grid(plan->tiles));
      e = plan->radix_bits == 10
              ? launch_chained(tile_hist_kernel<10>, hg, dim3(256), 0, s, a, plan->n, shift,
                               plan->tile, th, gs, nullptr, pp,
                               plan->tiles) : launch_chained(tile_hist_kernel<8>, hg, dim3(256), 0,
                               s, a, plan->n, shift, plan->tile, th, gs, nullptr, pp, plan->tiles);
      if (e != cudaSuccess) return e;
      e = launch_chained(tile_scan_split_kernel, dim3((plan->bins + 31) / 32, kScanSplits),
                         dim3(1024), 0, s, th, plan->tiles, plan->bins, base + p * plan->bins, pp,
                         gs);
      if (e != cudaSuccess) return e;
    }
    uint32_t* lb = lookback + (size_t)p * plan->tiles * plan->bins;
    e = launch_pass(*plan, p > 0, a, b, shift, base + p * plan->bins,
                    plan->cfg.scan == 0 ? lb : nullptr, counters + p, th, status, g, s, nullptr, 0,
                    da);
    if (e != cudaSuccess) return e;
    mark(rec, s);
    uint32_t* t = a;
    a = b;
    b = t;
  }
  *result = a;
  return cudaSuccess;
}

cudaError_t launch_sort_passes(uint32_t* keys, uint32_t* alt, const SortPlan* plan, void* ctrl,
                               uint32_t* status, cudaStream_t s, uint32_t** result,
                               Recorder* rec) {
  return sort_passes_impl(keys, alt, plan, ctrl, status, nullptr, s, result, rec);
}

cudaError_t launch_sort_passes_gated(uint32_t* keys, uint32_t* alt, const SortPlan* plan,
                                     void* ctrl, uint32_t* status, const uint32_t* gate,
                                     cudaStream_t s, uint32_t** result) {
  return sort_passes_impl(keys, alt, plan, ctrl, status, gate, s, result, nullptr);
}

cudaError_t launch_sort_passes_split(uint32_t* keys, uint32_t* alt, const SortPlan* plan,
                                     void* ctrl, uint32_t* status, const uint32_t* msd_flag,
                                     const uint32_t* lsd_flag, cudaStream_t s, uint32_t** result,
                                     Recorder* rec) {
  return sort_passes_impl(keys, alt, plan, ctrl, status, nullptr, s, result, rec, msd_flag,
                          lsd_flag);
}

bool msd_plan_ok(const SortPlan& p) {
  return p.radix_bits == 10 && p.passes == 3 && p.cfg.scan == 1;
}

cudaError_t launch_tile_hist(int radix_bits, const uint32_t* keys, int n, int shift,
                             const int4* tdesc, int tiles, uint32_t* th, cudaStream_t s,
                             const uint32_t* gate) {
  // a gated launch walks the tiles from a capped grid (few no-op CTAs)
  const int grid = gate ? tile_hist_grid(tiles) : tiles;
  if (radix_bits == 10)
    return launch_chained(tile_hist_kernel<10>, dim3(grid), dim3(256), 0, s, keys, n, shift, 0, th,
                          gate, tdesc, nullptr, tiles);
  return launch_chained(tile_hist_kernel<8>, dim3(grid), dim3(256), 0, s, keys, n, shift, 0, th,
                        gate, tdesc, nullptr, tiles);
}

}  // namespace octgb
