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
  constexpr int BINS = 1 << RB;
  extern __shared__ uint32_t s_hist[];
  if (HIST) {
    for (int i = threadIdx.x; i < passes * BINS; i += blockDim.x) s_hist[i] = 0;
    __syncthreads();
  }
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
      bad |= !(in_range(p[u].x, min_coord, range) && in_range(p[u].y, min_coord, range) &&
               in_range(p[u].z, min_coord, range));
      const uint32_t c = morton_code(p[u].x, p[u].y, p[u].z, min_coord, range);
      keys[i + u * stride] = c;
      if (HIST)
        for (int ps = 0; ps < passes; ++ps)
          atomicAdd(&s_hist[ps * BINS + ((c >> (ps * RB)) & (BINS - 1))], 1u);
    }
  }
  for (; i < n; i += stride) {
    const float4 p = ld_stream_f4(pts + i);
    bad |= !(in_range(p.x, min_coord, range) && in_range(p.y, min_coord, range) &&
             in_range(p.z, min_coord, range));
    const uint32_t c = morton_code(p.x, p.y, p.z, min_coord, range);
    keys[i] = c;
    if (HIST)
      for (int ps = 0; ps < passes; ++ps)
        atomicAdd(&s_hist[ps * BINS + ((c >> (ps * RB)) & (BINS - 1))], 1u);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) raise_status(status, kStatusRange);
  if (HIST) {
    for (int b = threadIdx.x; b < passes * BINS; b += blockDim.x)
      if (s_hist[b]) atomicAdd(&ghist[b], s_hist[b]);
  }
}

// --------------------------------------------------------------------------
// Digit histograms of existing keys (sort entry point without Morton).
// --------------------------------------------------------------------------
template <int RB>
__global__ void __launch_bounds__(256)
    histogram_kernel(const uint32_t* __restrict__ keys, int n, uint32_t* __restrict__ ghist,
                     int passes) {
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
                                                         uint32_t* __restrict__ base) {
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
// One OneSweep digit pass.
//   lookback[tile * BINS + b]: bits 31..30 flag (0 not ready, 1 tile count,
//   2 inclusive count of tiles 0..tile), bits 29..0 the count.
// --------------------------------------------------------------------------
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1;

template <int RB, int WARPS, int ITEMS>
struct PassSmem {
  static constexpr int BINS = 1 << RB;
  static constexpr int TILE = WARPS * 32 * ITEMS;
  static constexpr int HIST_BYTES = WARPS * BINS * 2;
  static constexpr int STAGE_BYTES = TILE * 4;
  static constexpr int UNION_BYTES = HIST_BYTES > STAGE_BYTES ? HIST_BYTES : STAGE_BYTES;
  static constexpr int BYTES = UNION_BYTES + BINS * 4 * 2 + 64 * 4;
};

template <int RB, int WARPS, int ITEMS>
__global__ void __launch_bounds__(WARPS * 32, 2)
    onesweep_pass_kernel(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int n,
                         int shift, const uint32_t* __restrict__ bin_base,
                         uint32_t* __restrict__ lookback, uint32_t* __restrict__ tile_counter,
                         uint32_t* __restrict__ status) {
  using L = PassSmem<RB, WARPS, ITEMS>;
  constexpr int BINS = L::BINS, THREADS = WARPS * 32, TILE = L::TILE;
  constexpr uint32_t MASK = BINS - 1;
  extern __shared__ __align__(16) unsigned char smem[];
  uint16_t* whist = reinterpret_cast<uint16_t*>(smem);  // [WARPS][BINS]
  uint32_t* stage = reinterpret_cast<uint32_t*>(smem);  // [TILE], aliases whist
  uint32_t* bin_local = reinterpret_cast<uint32_t*>(smem + L::UNION_BYTES);  // [BINS]
  uint32_t* bin_glob = bin_local + BINS;                                      // [BINS]
  uint32_t* misc = bin_glob + BINS;                                           // [64]

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) misc[0] = atomicAdd(tile_counter, 1u);
  for (int i = tid; i < WARPS * BINS / 2; i += THREADS) reinterpret_cast<uint32_t*>(whist)[i] = 0;
  __syncthreads();
  const int tile = (int)misc[0];
  const int tile_start = tile * TILE;
  const int valid = min(TILE, n - tile_start);

  // Load (warp-striped: item-major within each warp's contiguous segment).
  uint32_t key[ITEMS];
  const int wbase = tile_start + warp * 32 * ITEMS;
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    const int idx = wbase + it * 32 + lane;
    key[it] = idx < n ? __ldcs(src + idx) : 0xffffffffu;
  }

  // Warp multi-split ranking, stable in (item, lane) order.
  uint16_t rank[ITEMS];
  uint16_t* wh = whist + warp * BINS;
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    const uint32_t d = (key[it] >> shift) & MASK;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t before = wh[d];
    rank[it] = (uint16_t)(before + __popc(peers & lt));
    __syncwarp();
    if ((peers & lt) == 0) wh[d] = (uint16_t)(before + __popc(peers));
    __syncwarp();
  }
  __syncthreads();

  // Per-digit: exclusive offsets across warps, tile count, publish.
  const int invalid = TILE - valid;
  constexpr int PER_T = (BINS + THREADS - 1) / THREADS;
  uint32_t own[PER_T];
#pragma unroll
  for (int j = 0; j < PER_T; ++j) {
    const int b = tid + j * THREADS;
    if (b >= BINS) break;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t c = whist[w * BINS + b];
      whist[w * BINS + b] = (uint16_t)run;
      run += c;
    }
    bin_local[b] = run;  // tile count including out-of-range padding keys
    own[j] = run - (b == (int)MASK ? (uint32_t)invalid : 0u);
    st_release_u32(lookback + (size_t)tile * BINS + b, (tile == 0 ? kFlagInc : kFlagAgg) | own[j]);
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

  // Decoupled look-back per digit (bounded waits). The first probe reads the
  // immediate predecessor; past it, a thread loads a window of kWin
  // predecessor words at once (relaxed loads: flag and count share a word),
  // so walking back over k tiles that are not yet inclusive costs about
  // k / kWin round trips. Tiles that start together (the first wave) walk
  // far; later tiles usually stop at the first probe.
  constexpr int kWin = 16;
#pragma unroll
  for (int j = 0; j < PER_T; ++j) {
    const int b = tid + j * THREADS;
    if (b >= BINS) break;
    uint32_t prefix = 0;
    if (tile > 0) {
      int pred = tile - 1;
      uint32_t spins = 0;
      bool done = false;
      {  // first probe: the immediate predecessor
        uint32_t w0 = ld_relaxed_u32(lookback + (size_t)pred * BINS + b);
        while ((w0 & kFlagMask) == 0) {
          if (++spins > kSpinLimit) {
            raise_status(status, kStatusSpinTimeout);
            break;
          }
          backoff(spins);
          w0 = ld_relaxed_u32(lookback + (size_t)pred * BINS + b);
        }
        prefix += w0 & kValMask;
        done = (w0 & kFlagMask) == kFlagInc || spins > kSpinLimit;
        --pred;
      }
      while (!done) {
        uint32_t w[kWin];
#pragma unroll
        for (int k = 0; k < kWin; ++k)
          w[k] = (pred - k >= 0) ? ld_relaxed_u32(lookback + (size_t)(pred - k) * BINS + b)
                                 : kFlagInc;
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
        if (adv < kWin) {  // stopped at a word that is not ready yet: poll it again
          if (++spins > kSpinLimit) {
            raise_status(status, kStatusSpinTimeout);
            break;
          }
          backoff(spins);
        }
      }
      st_release_u32(lookback + (size_t)tile * BINS + b, kFlagInc | ((prefix + own[j]) & kValMask));
    }
    bin_glob[b] = bin_base[b] + prefix - bin_local[b];
  }

  // Local positions (read before the staging area overwrites the counters).
  uint16_t pos[ITEMS];
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    const uint32_t d = (key[it] >> shift) & MASK;
    pos[it] = (uint16_t)(bin_local[d] + whist[warp * BINS + d] + rank[it]);
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) stage[pos[it]] = key[it];
  __syncthreads();

  // Scatter in digit runs; padding keys sit at [valid, TILE) and are skipped.
#pragma unroll 4
  bool oob = false;
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

// --------------------------------------------------------------------------
// Host-side planning and launch.
// --------------------------------------------------------------------------
template <int RB, int WARPS, int ITEMS>
static int tiles_for(int n) {
  constexpr int TILE = WARPS * 32 * ITEMS;
  return (n + TILE - 1) / TILE;
}

SortPlan sort_plan(int n, int key_bits) {
  SortPlan p{};
  p.n = n;
  p.radix_bits = key_bits <= 30 ? 10 : 8;
  p.passes = (key_bits + p.radix_bits - 1) / p.radix_bits;
  if (p.passes < 1) p.passes = 1;
  p.bins = 1 << p.radix_bits;
  p.tile = p.radix_bits == 10 ? 16 * 32 * 16 : 16 * 32 * 15;
  p.tiles = n > 0 ? (n + p.tile - 1) / p.tile : 0;
  // control block: hist[passes*bins] + base[passes*bins] + counters[passes]
  // + lookback[passes*tiles*bins]
  p.hist_off = 0;
  p.base_off = align_up(p.hist_off + sizeof(uint32_t) * p.passes * p.bins, 256);
  p.counter_off = align_up(p.base_off + sizeof(uint32_t) * p.passes * p.bins, 256);
  p.lookback_off = align_up(p.counter_off + sizeof(uint32_t) * 64, 256);
  p.bytes = align_up(p.lookback_off + sizeof(uint32_t) * (size_t)p.passes * p.tiles * p.bins, 256);
  return p;
}

static int g_num_sms = 0;
int device_sm_count() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 152;
  }
  return g_num_sms;
}

template <int RB, int WARPS, int ITEMS>
static cudaError_t launch_pass(const uint32_t* src, uint32_t* dst, int n, int shift,
                               const uint32_t* base, uint32_t* lookback, uint32_t* counter,
                               uint32_t* status, cudaStream_t s) {
  using L = PassSmem<RB, WARPS, ITEMS>;
  auto k = onesweep_pass_kernel<RB, WARPS, ITEMS>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
    attr = true;
  }
  const int tiles = tiles_for<RB, WARPS, ITEMS>(n);
  k<<<tiles, WARPS * 32, L::BYTES, s>>>(src, dst, n, shift, base, lookback, counter, status);
  return cudaGetLastError();
}

cudaError_t launch_morton(const float4* pts, uint32_t* keys, long long n, float min_coord,
                          float range, const SortPlan* plan, void* ctrl, uint32_t* status,
                          cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int blocks = device_sm_count() * 4;
  long long need = (n + 255) / 256;
  const int grid = (int)(need < blocks ? need : blocks);
  if (plan) {
    uint32_t* hist = reinterpret_cast<uint32_t*>(static_cast<char*>(ctrl) + plan->hist_off);
    const size_t sm = sizeof(uint32_t) * plan->passes * plan->bins;
    if (plan->radix_bits == 10)
      morton_kernel<10, true><<<grid, 256, sm, s>>>(pts, keys, n, min_coord, range, hist,
                                                    plan->passes, status);
    else
      morton_kernel<8, true><<<grid, 256, sm, s>>>(pts, keys, n, min_coord, range, hist,
                                                   plan->passes, status);
  } else {
    morton_kernel<10, false><<<grid, 256, 0, s>>>(pts, keys, n, min_coord, range, nullptr, 0,
                                                  status);
  }
  return cudaGetLastError();
}

cudaError_t launch_histogram(const uint32_t* keys, const SortPlan* plan, void* ctrl,
                             cudaStream_t s) {
  if (plan->n <= 0) return cudaSuccess;
  uint32_t* hist = reinterpret_cast<uint32_t*>(static_cast<char*>(ctrl) + plan->hist_off);
  const size_t sm = sizeof(uint32_t) * plan->passes * plan->bins;
  const int blocks = device_sm_count() * 2;
  int need = (plan->n / 4 + 255) / 256 + 1;
  const int grid = need < blocks ? need : blocks;
  if (plan->radix_bits == 10)
    histogram_kernel<10><<<grid, 256, sm, s>>>(keys, plan->n, hist, plan->passes);
  else
    histogram_kernel<8><<<grid, 256, sm, s>>>(keys, plan->n, hist, plan->passes);
  return cudaGetLastError();
}

// Runs the digit passes (histograms must already be in the control block).
// Keys move src -> alt -> src ...; returns which buffer holds the result.
cudaError_t launch_sort_passes(uint32_t* keys, uint32_t* alt, const SortPlan* plan, void* ctrl,
                               uint32_t* status, cudaStream_t s, uint32_t** result,
                               Recorder* rec) {
  *result = keys;
  if (plan->n <= 1) return cudaSuccess;
  char* c = static_cast<char*>(ctrl);
  uint32_t* hist = reinterpret_cast<uint32_t*>(c + plan->hist_off);
  uint32_t* base = reinterpret_cast<uint32_t*>(c + plan->base_off);
  uint32_t* counters = reinterpret_cast<uint32_t*>(c + plan->counter_off);
  uint32_t* lookback = reinterpret_cast<uint32_t*>(c + plan->lookback_off);
  if (plan->radix_bits == 10)
    hist_scan_kernel<10><<<plan->passes, 1024, 0, s>>>(hist, base);
  else
    hist_scan_kernel<8><<<plan->passes, 256, 0, s>>>(hist, base);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  mark(rec, s);
  uint32_t* a = keys;
  uint32_t* b = alt;
  for (int p = 0; p < plan->passes; ++p) {
    uint32_t* lb = lookback + (size_t)p * plan->tiles * plan->bins;
    if (plan->radix_bits == 10)
      e = launch_pass<10, 16, 16>(a, b, plan->n, p * 10, base + p * plan->bins, lb, counters + p,
                                  status, s);
    else
      e = launch_pass<8, 16, 15>(a, b, plan->n, p * 8, base + p * plan->bins, lb, counters + p,
                                 status, s);
    if (e != cudaSuccess) return e;
    mark(rec, s);
    uint32_t* t = a;
    a = b;
    b = t;
  }
  *result = a;
  return cudaSuccess;
}

}  // namespace octgb
