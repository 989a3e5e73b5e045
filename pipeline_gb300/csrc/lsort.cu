// Learned bucketed sort + unique (stages 2-3 driven by the learned CDF).
//
// With a model whose bucket(v) never decreases with v, sorting reduces to a
// scatter into buckets followed by an independent sort of each bucket, and the
// unique pass fuses into the bucket stage (equal keys share a bucket):
//
//   bin      one pass over the points (or keys): Morton code, bucket, and a
//            place in the bucket's fixed range of cap keys, reserved per
//            tile and bucket on the bucket's cursor (see the bin section)
//   stats    bucket counts from the cursors; overflow fraction (keys in
//            buckets above the bitonic capacity) and the fallback decision
//            (a bucket past cap, or the fraction above the threshold)
//   buckets  one CTA per bucket: the sorted unique keys of the bucket from a
//            shared-memory bitmap over [min, max] of its keys when that is
//            dense enough, else a radix sort (or, above the cache size, a
//            bitonic sort) of its keys in shared memory; the run overwrites
//            the front of the bucket's own range, its length goes to a table
//   pack     a scan of the run lengths and one copy per bucket assemble the
//            output (no bucket ever waits on another)
//
// Bucket ids come from the model's boundary table (the smallest key of every
// bucket) narrowed by a 2^14-entry table over the top key bits, both staged
// in shared memory; that is the model's own fixed-point bucket function,
// evaluated without its per-key knot search and 64-bit multiply.
//
// If any bucket fits neither form, the overflow fraction exceeds the
// threshold, or the model's tables were built for another bucket count, the
// device flag `fallback` is set and the OneSweep sort + unique (launched right
// after, gated on the flag) redo stages 2-3 from the original keys; otherwise
// those launches return at once. Either way the output is the sorted unique
// key array, identical to the plain path's.
#include <stdio.h>

#include <algorithm>

#include "learned.cuh"
#include "lsort.cuh"

namespace octgb {

constexpr int kBkThreads = 512;           // bucket CTAs (3 per SM)
constexpr int kBkWarps = kBkThreads / 32;
constexpr int kBkWords = 16384;           // 64 KiB working region per bucket CTA
constexpr int kBkCache = 8192;            // keys cached in the first half (cnt <= kBkCache)
constexpr int kBkItems = kBkCache / kBkThreads;  // keys per thread in the radix sort
constexpr uint32_t kBmSmall = 1u << 18;   // bitmap span in the second half (32 KiB)
constexpr uint32_t kBmBig = 1u << 19;     // bitmap span over the whole region (64 KiB)
constexpr int kCap = kBkWords;            // bitonic capacity (keys)
constexpr int kRsBits = 8;                // radix-sort digit width
constexpr int kRsBins = 1 << kRsBits;

// ------------------------------------------------------- bucket lookup --
struct BucketLookup {
  const uint32_t* bounds;  // [nb] smallest key of each bucket (shared memory)
  const uint16_t* blut;    // [2^14 + 1] bucket at the start of each 2^16-key cell (shared,
                           // 4-byte aligned)
  uint32_t last;           // nb - 1
};

// Stage the lookup tables in shared memory (all threads; ends with a barrier).
__device__ __forceinline__ BucketLookup load_lookup(const char* __restrict__ blob,
                                                    const LcdfLayout& L, int nb,
                                                    uint32_t* s_bounds, uint16_t* s_blut) {
  const uint32_t* gb = reinterpret_cast<const uint32_t*>(blob + L.bounds);
  const uint32_t* gl = reinterpret_cast<const uint32_t*>(blob + L.blut);
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s_bounds[b] = gb[b];
  uint32_t* sl = reinterpret_cast<uint32_t*>(s_blut);
  for (int p = threadIdx.x; p < kLcdfBlutSize / 2; p += blockDim.x) sl[p] = gl[p];
  if (threadIdx.x == 0)
    s_blut[kLcdfBlutSize] = reinterpret_cast<const uint16_t*>(blob + L.blut)[kLcdfBlutSize];
  __syncthreads();
  return BucketLookup{s_bounds, s_blut, (uint32_t)(nb - 1)};
}

// bucket(v): the largest b with bounds[b] <= v, searched in
// [blut[v >> 16], blut[(v >> 16) + 1]], clamped to nb - 1.
__device__ __forceinline__ uint32_t bucket_of(const BucketLookup& q, uint32_t v) {
  const uint32_t vc = min(v, kLcdfKeyEnd - 1u);
  const uint32_t p = vc >> (30 - kLcdfBlutBits);
  uint32_t hi = min((uint32_t)q.blut[p + 1], q.last);
  uint32_t lo = min((uint32_t)q.blut[p], hi);
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (q.bounds[mid] <= vc) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Shared memory of the batched histogram and scatter kernels: counts or
// cursors [nb], bounds [nb], the bucket table [2^14 + 1].
size_t lsort_hist_smem(int nb, int /*max_segments*/) {
  return align_up(8 * (size_t)nb + 2 * ((size_t)kLcdfBlutSize + 2), 16);
}

// ------------------------------------------------------------------- bin --
// One pass over the points (or keys) does what a histogram pass and a
// scatter pass would: the Morton code, its bucket and its place in the
// bucket. Bucket b owns the fixed range [b * cap, (b + 1) * cap) of bkeys.
// CTAs (one per SM) walk tiles of up to kBinTile keys (their length chosen so
// that every CTA gets the same number of tiles): shared-memory atomics rank a
// tile's keys per bucket, one atomicAdd on the bucket's cursor reserves each
// bucket's run, the keys are staged in bucket order and leave bucket by
// bucket, so the runs that consecutive tiles write into a bucket lie next to
// each other. A bucket that outgrows cap drops the keys past it; its cursor
// still counts them, which sends the sort to the fallback.
// One 1,024-thread CTA per SM: two 512-thread CTAs with 4,096-key tiles
// measured 9% slower on the learned build (twice the cursor atomics per key).
constexpr int kBinCtasPerSm = 1;
constexpr int kBinThreads = 1024 / kBinCtasPerSm;
// 16 keys per thread: a 16,384-key tile halves the cursor atomics per key
// against 8,192 keys (learned build 0.872 vs 0.902 ms from a graph, 16.7M
// clustered points); its 96 KiB stage is the largest that fits beside the tables.
constexpr int kBinItems = 16;
constexpr int kBinTile = kBinThreads * kBinItems;  // 16,384 keys
static_assert(kBinTile <= 32768, "ranks are kept in 15 bits");

// counts (then run bases), local starts and bounds [nb] each, the Morton
// spread table [1024], the staged keys [kBinTile] and their buckets, the
// bucket table
size_t lsort_bin_smem(int nb) {
  return align_up(12 * (size_t)nb + 4 * 1024 + 6 * (size_t)kBinTile +
                      2 * ((size_t)kLcdfBlutSize + 2),
                  16);
}

template <bool FROM_POINTS>
__global__ void __launch_bounds__(kBinThreads, kBinCtasPerSm)
    lsort_bin_kernel(const float4* __restrict__ pts, uint32_t* __restrict__ keys, int n,
                     float min_coord, float range, const char* __restrict__ blob, LcdfLayout L,
                     int nb, uint32_t cap, int tile, uint32_t* __restrict__ cursor,
                     uint32_t* __restrict__ bkeys, uint32_t* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t total;
  uint32_t* s_cnt = reinterpret_cast<uint32_t*>(sm);
  uint32_t* s_gbase = s_cnt;  // a bucket's count becomes its run base once the run is reserved
  uint32_t* s_lstart = s_cnt + nb;
  uint32_t* s_bounds = s_lstart + nb;
  uint32_t* spread = s_bounds + nb;
  uint32_t* st_key = spread + 1024;
  uint16_t* st_bid = reinterpret_cast<uint16_t*>(st_key + kBinTile);
  uint16_t* s_coarse = st_bid + kBinTile;
  if (FROM_POINTS) fill_spread_lut(spread);
  const BucketLookup q = load_lookup(blob, L, nb, s_bounds, s_coarse);
  const float scale = __fdiv_rn(1024.0f, range);
  const int tid = threadIdx.x;
  // tile in [1, kBinTile]: thread tid takes positions it * kBinThreads + tid
  // of its tile; those below the tile's end are a prefix of each warp
  const int tiles = (n + tile - 1) / tile;
  const int per = (nb + kBinThreads - 1) / kBinThreads;  // buckets per thread in the scan
  bool bad = false;
  for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
    for (int b = tid; b < nb; b += kBinThreads) s_cnt[b] = 0;
    __syncthreads();
    const int t0 = t * tile;
    const int t_end = min(n, t0 + tile);
    uint32_t code[kBinItems], br[kBinItems];  // code; bucket << 16 | rank in the bucket
#pragma unroll
    for (int h = 0; h < kBinItems; h += 4) {
      float4 p[4];
      uint32_t kk[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = t0 + (h + u) * kBinThreads + tid;
        const bool in = i < t_end;
        if (FROM_POINTS) {
          if (in) p[u] = ld_stream_f4(pts + i);
        } else {
          kk[u] = in ? __ldcs(keys + i) : 0u;
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = t0 + (h + u) * kBinThreads + tid;
        code[h + u] = 0;
        br[h + u] = 0;
        if (i < t_end) {
          uint32_t c;
          if (FROM_POINTS) {
            bool ok;
            c = morton_code_lut(p[u].x, p[u].y, p[u].z, min_coord, range, scale, spread, ok);
            bad |= !ok;
            keys[i] = c;  // the fallback sorts these
          } else {
            c = kk[u];
          }
          code[h + u] = c;
        }
        // Only unique keys are needed: a key equal to the previous lane's
        // (the key before it) stays out of the buckets, so runs of one cell
        // (scan-ordered clouds) shrink before the buckets see them. Lanes
        // hold consecutive keys and the valid ones are a prefix of the warp.
        const uint32_t prev = __shfl_up_sync(0xffffffffu, code[h + u], 1);
        if (i < t_end && ((tid & 31) == 0 || prev != code[h + u])) {
          const uint32_t b = bucket_of(q, code[h + u]);
          br[h + u] = (b << 16) | atomicAdd(&s_cnt[b], 1u) | 0x8000u;  // bit 15: placed
        }
      }
    }
    __syncthreads();
    // Local starts (exclusive scan over buckets); each bucket's run reserved.
    int placed;  // keys of the tile that go to buckets
    {
      const int b0 = tid * per, b1 = min(b0 + per, nb);
      uint32_t sum = 0;
      for (int b = b0; b < b1; ++b) sum += s_cnt[b];
      uint32_t run = block_exclusive_sum<kBinThreads>(sum, warp_tot, &total);
      placed = (int)total;
      // four buckets at a time: their cursor atomics are in flight together
      for (int b = b0; b < b1; b += 4) {
        uint32_t c[4], g[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) c[k] = b + k < b1 ? s_cnt[b + k] : 0u;
#pragma unroll
        for (int k = 0; k < 4; ++k) g[k] = c[k] ? atomicAdd(cursor + b + k, c[k]) : 0u;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (b + k < b1) {
            s_lstart[b + k] = run;
            s_gbase[b + k] = g[k] - run;  // tile position j of the bucket goes to slot s_gbase + j
            run += c[k];
          }
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kBinItems; ++it) {
      if (br[it] & 0x8000u) {
        const uint32_t b = br[it] >> 16;
        const uint32_t pos = s_lstart[b] + (br[it] & 0x7fffu);
        st_key[pos] = code[it];
        st_bid[pos] = (uint16_t)b;
      }
    }
    __syncthreads();
    for (int j = tid; j < placed; j += kBinThreads) {
      const uint32_t b = st_bid[j];
      const uint32_t o = s_gbase[b] + (uint32_t)j;
      if (o < cap) bkeys[(size_t)b * cap + o] = st_key[j];
    }
    __syncthreads();  // the stage and counters are the next tile's
  }
  if (FROM_POINTS && __syncthreads_or(bad) && tid == 0) raise_status(status, kStatusRange);
}

// One block: bucket totals from the cursors, the fixed bucket starts
// (b * cap), overflow fraction and the fallback decision (a bucket past cap,
// too many keys in buckets above the bitonic capacity, or tables built for
// another bucket count).
__global__ void __launch_bounds__(1024)
    lsort_bin_stats_kernel(const uint32_t* __restrict__ cursor, int nb, int n, uint32_t cap,
                           float threshold, const char* __restrict__ blob,
                           uint32_t* __restrict__ starts, uint32_t* __restrict__ counts,
                           LsortStats* __restrict__ stats) {
  __shared__ uint32_t s_over, s_max, s_spill;
  if (threadIdx.x == 0) {
    s_over = 0;
    s_max = 0;
    s_spill = 0;
  }
  __syncthreads();
  uint32_t over = 0, mx = 0, spill = 0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const uint32_t v = cursor[b];
    if (v > (uint32_t)kCap) over += v;
    if (v > cap) spill = 1u;
    mx = max(mx, v);
    starts[b] = (uint32_t)b * cap;
    counts[b] = min(v, cap);
  }
  atomicAdd(&s_over, over);
  atomicMax(&s_max, mx);
  if (spill) atomicOr(&s_spill, 1u);
  __syncthreads();
  if (threadIdx.x == 0) {
    starts[nb] = (uint32_t)nb * cap;
    stats->overflow_keys = s_over;
    stats->max_bucket = s_max;
    stats->n = (uint32_t)n;
    const float frac = n > 0 ? (float)s_over / (float)n : 0.f;
    stats->overflow_frac = frac;
    const LcdfHeader* h = reinterpret_cast<const LcdfHeader*>(blob);
    const bool model_ok = h->magic == kLcdfMagic && h->version == kLcdfVersion &&
                          h->n_buckets == nb;
    if (frac > threshold || !model_ok || s_spill) {
      stats->skip = 1u;
      stats->fallback = 1u;
    }
  }
}

// ---------------------------------------------------------------- buckets --
struct BucketSmem {
  uint32_t buf[kBkWords];  // keys cache + bitmap or radix ping-pong, whole-region bitmap, or bitonic keys
  uint16_t whist[kBkWarps][kRsBins];  // radix sort: per-warp digit counts, then offsets
  uint32_t dstart[kRsBins];           // radix sort: first position of each digit
  uint32_t red[2][kBkWarps];
  uint32_t warp_base[32];
  uint32_t misc[8];
};

// Stable LSD radix sort of a[0, cnt) (cnt <= kBkCache) on the low `bits`
// bits of key - kmin, 8-bit digits, ping-pong between a and b. Warp w ranks
// its contiguous kBkItems * 32 keys with ballot multi-split (peers = lanes
// with the same digit), so ties keep input order. Returns the sorted array.
__device__ uint32_t* bucket_radix_sort(uint32_t* a, uint32_t* b, int cnt, uint32_t kmin, int bits,
                                       BucketSmem& S) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const uint32_t lt = lanemask_lt();
  // every warp takes `items` rows of 32 keys (the last warps may be partial)
  const int items = (cnt + kBkWarps * 32 - 1) / (kBkWarps * 32);
  const int seg = items * 32;
  // peers from two 4-bit half-digit equality tables (lane v: lanes whose half
  // equals v), fetched by shuffle
  constexpr int kHalf = kRsBits / 2;
  uint32_t lane_bits[kHalf];
#pragma unroll
  for (int b = 0; b < kHalf; ++b) lane_bits[b] = 0u - ((uint32_t)(lane >> b) & 1u);
  for (int shift = 0; shift < bits; shift += kRsBits) {
    for (int k = tid; k < kBkWarps * kRsBins / 2; k += kBkThreads)
      reinterpret_cast<uint32_t*>(S.whist)[k] = 0;
    __syncthreads();
    uint32_t rk[kBkItems / 2];  // two 16-bit ranks per register; keys are re-read
    uint16_t* wh = S.whist[wid];
    if (shift == 0) {
      // The first pass needs no stability (the bucket's keys arrive in any
      // order): a shared-memory atomic on the warp's 16-bit digit counter
      // (the upper or lower half of its 32-bit word; a warp counts at most
      // kBkItems * 32 keys, so no carry reaches the other half) ranks a key.
      uint32_t* wh32 = reinterpret_cast<uint32_t*>(wh);
#pragma unroll
      for (int it = 0; it < kBkItems; ++it) {
        if (it >= items) break;
        const int idx = wid * seg + it * 32 + lane;
        uint32_t r = 0;
        if (idx < cnt) {
          const uint32_t dg = (a[idx] - kmin) & (kRsBins - 1);
          const uint32_t sh = 16u * (dg & 1u);
          r = (atomicAdd(&wh32[dg >> 1], 1u << sh) >> sh) & 0xffffu;
        }
        if (it & 1) rk[it >> 1] |= r << 16;
        else rk[it >> 1] = r;
      }
    } else {
#pragma unroll
      for (int it = 0; it < kBkItems; ++it) {
        if (it >= items) break;
        const int idx = wid * seg + it * 32 + lane;
        const bool valid = idx < cnt;
        const uint32_t key = valid ? a[idx] : 0u;
        const uint32_t dg = ((key - kmin) >> shift) & (kRsBins - 1);
        uint32_t eq_lo = 0xffffffffu, eq_hi = 0xffffffffu;
#pragma unroll
        for (int bit = 0; bit < kHalf; ++bit) {
          eq_lo &= ~(__ballot_sync(0xffffffffu, (dg >> bit) & 1u) ^ lane_bits[bit]);
          eq_hi &= ~(__ballot_sync(0xffffffffu, (dg >> (kHalf + bit)) & 1u) ^ lane_bits[bit]);
        }
        const uint32_t peers = __ballot_sync(0xffffffffu, valid) &
                               __shfl_sync(0xffffffffu, eq_lo, (int)(dg & ((1u << kHalf) - 1u))) &
                               __shfl_sync(0xffffffffu, eq_hi, (int)(dg >> kHalf));
        const uint32_t before = valid ? wh[dg] : 0u;
        const uint32_t r = before + __popc(peers & lt);
        if (it & 1) rk[it >> 1] |= r << 16;
        else rk[it >> 1] = r;
        __syncwarp();
        if (valid && (peers & lt) == 0) wh[dg] = (uint16_t)(before + __popc(peers));
        __syncwarp();
      }
    }
    __syncthreads();
    // per digit: exclusive offsets over warps, then digit starts over digits
    uint32_t tot = 0;
    if (tid < kRsBins) {
#pragma unroll
      for (int w = 0; w < kBkWarps; ++w) {
        const uint32_t c = S.whist[w][tid];
        S.whist[w][tid] = (uint16_t)tot;
        tot += c;
      }
    }
    const uint32_t start = block_exclusive_sum<kBkThreads>(tid < kRsBins ? tot : 0u, S.warp_base,
                                                           &S.misc[5]);
    if (tid < kRsBins) S.dstart[tid] = start;
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kBkItems; ++it) {
      if (it >= items) break;
      const int idx = wid * seg + it * 32 + lane;
      if (idx < cnt) {
        const uint32_t key = a[idx];
        const uint32_t dg = ((key - kmin) >> shift) & (kRsBins - 1);
        const uint32_t r = (rk[it >> 1] >> ((it & 1) * 16)) & 0xffffu;
        b[S.dstart[dg] + S.whist[wid][dg] + r] = key;
      }
    }
    __syncthreads();
    uint32_t* t = a;
    a = b;
    b = t;
  }
  return a;
}

// Bitmap words [seg0, seg1) of this warp: lanes take consecutive words.
// Pass 0 returns the warp's popcount; pass 1 emits keys at base + rank, into
// shared memory (stage) or global memory.
__device__ __forceinline__ uint32_t bitmap_emit(const uint32_t* bm, int seg0, int seg1,
                                                uint32_t kmin, bool emit, uint32_t base,
                                                uint32_t* dst) {
  const int lane = threadIdx.x & 31;
  uint32_t run = 0;
  for (int w0 = seg0; w0 < seg1; w0 += 32) {
    const int w = w0 + lane;
    uint32_t bits = w < seg1 ? bm[w] : 0u;
    const uint32_t c = __popc(bits);
    uint32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (emit) {
      uint32_t pos = base + run + inc - c;
      const uint32_t kw = kmin + ((uint32_t)w << 5);
      while (bits) {
        const int bit = __ffs(bits) - 1;
        bits &= bits - 1;
        dst[pos++] = kw + (uint32_t)bit;
      }
    }
    run += __shfl_sync(0xffffffffu, inc, 31);
  }
  return run;
}

// Sorted keys a[seg0, seg1) of this warp (a[-1] read for run heads).
__device__ __forceinline__ uint32_t heads_emit(const uint32_t* a, int seg0, int seg1, bool emit,
                                               uint32_t base, uint32_t* dst) {
  const int lane = threadIdx.x & 31;
  uint32_t run = 0;
  for (int i0 = seg0; i0 < seg1; i0 += 32) {
    const int i = i0 + lane;
    const bool head = i < seg1 && (i == 0 || a[i] != a[i - 1]);
    const uint32_t m = __ballot_sync(0xffffffffu, head);
    if (emit && head) dst[base + run + __popc(m & lanemask_lt())] = a[i];
    run += __popc(m);
  }
  return run;
}

// One CTA per bucket: the bucket's sorted unique keys overwrite the front of
// its own range of bkeys (its keys are in shared memory, or in the bitmap,
// by then) and its unique count goes to ucount[b]; buckets never wait on one
// another. A scan of the counts and a copy kernel then pack the runs.
__global__ void __launch_bounds__(kBkThreads, 3)
    lsort_bucket_kernel(uint32_t* __restrict__ bkeys, const uint32_t* __restrict__ starts,
                        uint32_t* __restrict__ ucount, LsortStats* __restrict__ stats,
                        const uint32_t* __restrict__ counts = nullptr) {
  // `skip` is final before this kernel starts; `fallback` may still be set by
  // a failing bucket.
  if (stats->skip) return;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  BucketSmem& S = *reinterpret_cast<BucketSmem*>(sm_raw);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int b = blockIdx.x;
  // bucket b: keys [starts[b], starts[b] + counts[b]), or up to starts[b + 1]
  const uint32_t lo = starts[b];
  const int cnt = (int)(counts ? counts[b] : starts[b + 1] - lo);
  const bool cached = cnt <= kBkCache;
  // keys -> cache, and the key span of the bucket (four loads per thread in
  // flight)
  uint32_t kmin = 0xffffffffu, kmax = 0;
  for (int i0 = tid; i0 < cnt; i0 += 4 * kBkThreads) {
    uint32_t k[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * kBkThreads;
      k[u] = i < cnt ? bkeys[lo + i] : 0u;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * kBkThreads;
      if (i < cnt) {
        if (cached) S.buf[i] = k[u];
        kmin = min(kmin, k[u]);
        kmax = max(kmax, k[u]);
      }
    }
  }
  kmin = __reduce_min_sync(0xffffffffu, kmin);
  kmax = __reduce_max_sync(0xffffffffu, kmax);
  if (lane == 0) {
    S.red[0][wid] = kmin;
    S.red[1][wid] = kmax;
  }
  __syncthreads();
  if (wid == 0) {
    uint32_t a = lane < kBkWarps ? S.red[0][lane] : 0xffffffffu;
    uint32_t z = lane < kBkWarps ? S.red[1][lane] : 0u;
    a = __reduce_min_sync(0xffffffffu, a);
    z = __reduce_max_sync(0xffffffffu, z);
    if (lane == 0) {
      S.misc[1] = a;
      S.misc[2] = z;
    }
  }
  __syncthreads();
  kmin = S.misc[1];
  kmax = S.misc[2];
  const uint32_t span_m1 = cnt > 0 ? kmax - kmin : 0u;  // span - 1

  // 0: bitmap in the second half, keys cached in the first (output staged);
  //    taken while the bitmap has at most 4 words per key (dense buckets)
  // 1: bitmap over the whole region (keys re-read, output written directly):
  //    buckets above the cache size, or cached ones that are as dense but
  //    span more than the second half
  // 2: sorted keys: radix sort of the cached keys (cnt <= kBkCache) or
  //    bitonic sort of up to kCap keys over the whole region
  // 3: neither fits
  // Walking a bitmap word costs a few instructions where ranking a key costs
  // tens per 8-bit pass (2-3 passes for these spans): up to 4 words per key
  // the bitmap is cheaper.
  const uint32_t words_needed = (span_m1 >> 5) + 1u;
  const bool dense = words_needed <= max(4u * (uint32_t)cnt, 256u);
  int path;
  bool radix = false;
  if (cnt == 0) {
    path = 0;
  } else if (cached) {
    if (span_m1 < kBmSmall && dense) {
      path = 0;
    } else if (span_m1 < kBmBig && dense) {
      path = 1;
    } else {
      path = 2;
      radix = true;
    }
  } else if (span_m1 < kBmBig) {
    path = 1;
  } else if (cnt <= kCap) {
    path = 2;
  } else {
    path = 3;
  }
  if (tid == 0 && cnt > 0)
    atomicAdd(path <= 1 ? &stats->bitmap_buckets
                        : path == 3 ? &stats->failed_buckets
                                    : radix ? &stats->radix_buckets : &stats->bitonic_buckets,
              1u);

  uint32_t* bm = path == 0 ? S.buf + kBkCache : S.buf;
  uint32_t* sorted = S.buf;
  const int words = (path <= 1 && cnt > 0) ? (int)words_needed : 0;
  int n_items = 0;  // bitmap words or sorted keys walked by the count/emit passes
  if (path <= 1) {
    for (int w = tid; w < words; w += kBkThreads) bm[w] = 0;
    __syncthreads();
    if (path == 0) {
      for (int i = tid; i < cnt; i += kBkThreads) {
        const uint32_t r = S.buf[i] - kmin;
        atomicOr(&bm[r >> 5], 1u << (r & 31));
      }
    } else {
      for (int i0 = tid; i0 < cnt; i0 += 4 * kBkThreads) {
        uint32_t k[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = i0 + u * kBkThreads;
          k[u] = i < cnt ? bkeys[lo + i] : 0u;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (i0 + u * kBkThreads < cnt) {
            const uint32_t r = k[u] - kmin;
            atomicOr(&bm[r >> 5], 1u << (r & 31));
          }
        }
      }
    }
    __syncthreads();
    n_items = words;
  } else if (path == 2 && radix) {
    const int bits = 32 - __clz(span_m1);
    sorted = bucket_radix_sort(S.buf, S.buf + kBkCache, cnt, kmin, bits, S);
    n_items = cnt;
  } else if (path == 2) {
    int m = 1;
    while (m < cnt) m <<= 1;
    for (int i = tid; i < m; i += kBkThreads) S.buf[i] = i < cnt ? bkeys[lo + i] : 0xffffffffu;
    __syncthreads();
    // bitonic network over m keys; each thread takes m / 2 / kBkThreads pairs
    for (int k = 2; k <= m; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int p = tid; p < (m >> 1); p += kBkThreads) {
          const int i = ((p & ~(j - 1)) << 1) | (p & (j - 1));
          const uint32_t a = S.buf[i], c = S.buf[i + j];
          if ((a > c) == ((i & k) == 0)) {
            S.buf[i] = c;
            S.buf[i + j] = a;
          }
        }
        __syncthreads();
      }
    }
    n_items = cnt;
  } else if (tid == 0) {
    atomicOr(&stats->fallback, 1u);
  }

  // Warp segments of the walked items: count, scan over warps, emit.
  const int per_warp = ((n_items + kBkWarps - 1) / kBkWarps + 31) & ~31;
  const int seg0 = min(wid * per_warp, n_items), seg1 = min(seg0 + per_warp, n_items);
  uint32_t wcount = 0;
  if (path <= 1) wcount = bitmap_emit(bm, seg0, seg1, kmin, false, 0, nullptr);
  else if (path == 2) wcount = heads_emit(sorted, seg0, seg1, false, 0, nullptr);
  if (lane == 0) S.warp_base[wid] = wcount;
  __syncthreads();
  if (wid == 0) {
    const uint32_t x = lane < kBkWarps ? S.warp_base[lane] : 0u;
    uint32_t inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane < kBkWarps) S.warp_base[lane] = inc - x;
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    if (lane == 0) S.misc[3] = path == 3 ? 0u : total;
  }
  __syncthreads();
  const uint32_t uniq = S.misc[3];
  const uint32_t wbase = S.warp_base[wid];
  uint32_t* dst = bkeys + lo;
  if (path == 0 && uniq > 0) {
    // stage the bucket's unique keys over the key cache, then copy out coalesced
    bitmap_emit(bm, seg0, seg1, kmin, true, wbase, S.buf);
    __syncthreads();
    for (uint32_t i = tid; i < uniq; i += kBkThreads) dst[i] = S.buf[i];
  } else if (path == 1) {
    bitmap_emit(bm, seg0, seg1, kmin, true, wbase, dst);
  } else if (path == 2) {
    heads_emit(sorted, seg0, seg1, true, wbase, dst);
  }
  if (tid == 0) ucount[b] = uniq;
}

// One block: exclusive scan of the per-bucket unique counts; U to *d_unique.
__global__ void __launch_bounds__(1024)
    lsort_uscan_kernel(const uint32_t* __restrict__ ucount, int nb, uint32_t* __restrict__ uoff,
                       int* __restrict__ d_unique, const LsortStats* __restrict__ stats) {
  if (stats->fallback) return;  // final once the bucket kernel is done
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t total;
  const int per = (nb + 1023) / 1024;
  uint32_t sum = 0;
  for (int j = 0; j < per; ++j) {
    const int b = threadIdx.x * per + j;
    if (b < nb) sum += ucount[b];
  }
  uint32_t run = block_exclusive_sum<1024>(sum, warp_tot, &total);
  for (int j = 0; j < per; ++j) {
    const int b = threadIdx.x * per + j;
    if (b < nb) {
      uoff[b] = run;
      run += ucount[b];
    }
  }
  if (threadIdx.x == 0) *d_unique = (int)total;
}

// dst[0, n) = src[0, n) by the whole block, four loads per thread in flight.
__device__ __forceinline__ void copy_run(uint32_t* __restrict__ dst,
                                         const uint32_t* __restrict__ src, uint32_t n) {
  constexpr int U = 4;
  const uint32_t step = blockDim.x * U;
  for (uint32_t i0 = threadIdx.x; i0 < n; i0 += step) {
    uint32_t v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t i = i0 + (uint32_t)u * blockDim.x;
      if (i < n) v[u] = src[i];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t i = i0 + (uint32_t)u * blockDim.x;
      if (i < n) dst[i] = v[u];
    }
  }
}

// One block per bucket: its unique run, from the front of its bkeys range to
// its place in the output.
__global__ void __launch_bounds__(256)
    lsort_compact_kernel(const uint32_t* __restrict__ bkeys, const uint32_t* __restrict__ starts,
                         const uint32_t* __restrict__ ucount, const uint32_t* __restrict__ uoff,
                         uint32_t* __restrict__ out, const LsortStats* __restrict__ stats) {
  if (stats->fallback) return;
  const int b = blockIdx.x;
  copy_run(out + uoff[b], bkeys + starts[b], ucount[b]);
}

// ----------------------------------------------------- batched learned sort --
// The clouds of a batch share one model over their own (per-cloud
// quantised) Morton codes. Bucket b of cloud c holds the cloud's keys with
// bucket(key) == b, so the unique keys of each cloud's buckets, in bucket
// order, are the cloud's sorted unique keys:
//   lb_hist      per sort tile (tiles never cross clouds): bucket counts of
//                the keys left after dropping repeats within each warp's 32
//   lb_scan      per cloud: every tile's offset in every bucket, bucket starts
//   lb_scatter   per tile: each of those keys to its bucket (any order)
//   lsort_bucket one CTA per (cloud, bucket), the single-cloud bucket kernel:
//                the bucket's sorted unique keys at its front (bitmap, radix
//                or bitonic form); a bucket that fits no form sets fallback
//   lb_uscan     per cloud: offsets of the buckets' unique runs
//   lb_compact   the runs, packed per cloud at the cloud's start
//   lb_pad       the rest of each cloud's range filled with its largest key,
//                so the cloud's range holds sorted keys (its unique keys,
//                then copies of the last one) for the batched unique stage
// With fallback set, the last three return at once and the plain LSD passes
// (gated on the same flag) sort the original keys instead.
// Only the unique keys of each cloud are needed, so of the equal keys among
// a warp's 32 consecutive keys (in scan order) only the lowest lane's goes to
// a bucket: dense clusters (many points in one cell) shrink before the
// buckets see them. The histogram and the scatter group the keys the same
// way, so their counts agree. Lanes past the tile hold 2^32 - 1, which no
// code reaches.
__device__ __forceinline__ bool lb_first_of_its_key(uint32_t k) {
  const uint32_t peers = __match_any_sync(0xffffffffu, k);
  return k != 0xffffffffu && (peers & lanemask_lt()) == 0;
}

// CTAs walk the tiles from a capped grid, so each stages the model's lookup
// tables once for several tiles. A warp takes kLbRows rows of 32 consecutive
// keys at a time (their loads in flight together); rows start at the tile's
// first key + 32 r in both kernels, so both drop the same repeats.
constexpr int kLbRows = 4;

__global__ void __launch_bounds__(256)
    lb_hist_kernel(const uint32_t* __restrict__ keys, const int4* __restrict__ tiles, int n_tiles,
                   const char* __restrict__ blob, LcdfLayout L, int nb,
                   uint32_t* __restrict__ tile_off) {
  extern __shared__ __align__(16) unsigned char sm[];
  uint32_t* s_hist = reinterpret_cast<uint32_t*>(sm);
  const BucketLookup q =
      load_lookup(blob, L, nb, s_hist + nb, reinterpret_cast<uint16_t*>(s_hist + 2 * nb));
  const int lane = threadIdx.x & 31;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s_hist[b] = 0;
    __syncthreads();
    const int4 d = tiles[t];
    for (int base = d.x + (int)(threadIdx.x >> 5) * 32 * kLbRows; base < d.y;
         base += blockDim.x * kLbRows) {
      uint32_t k[kLbRows];
#pragma unroll
      for (int u = 0; u < kLbRows; ++u) {
        const int i = base + u * 32 + lane;
        k[u] = i < d.y ? keys[i] : 0xffffffffu;  // no code reaches 2^32 - 1
      }
#pragma unroll
      for (int u = 0; u < kLbRows; ++u)
        if (lb_first_of_its_key(k[u])) atomicAdd(&s_hist[bucket_of(q, k[u])], 1u);
    }
    __syncthreads();
    uint32_t* row = tile_off + (size_t)t * nb;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) row[b] = s_hist[b];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(1024)
    lb_scan_kernel(const int* __restrict__ start, const int* __restrict__ cloud_tile0, int nb,
                   int C, uint32_t* __restrict__ tile_off, uint32_t* __restrict__ bstart,
                   uint32_t* __restrict__ bcount, LsortStats* __restrict__ stats) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  extern __shared__ __align__(16) unsigned char sm[];
  uint32_t* tot = reinterpret_cast<uint32_t*>(sm);
  const int c = blockIdx.x;
  const int t0 = cloud_tile0[c], t1 = cloud_tile0[c + 1];
  // per bucket: offsets of the cloud's tiles inside the bucket (column scan)
  uint32_t big = 0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    uint32_t run = 0;
    for (int t = t0; t < t1; ++t) {
      const uint32_t v = tile_off[(size_t)t * nb + b];
      tile_off[(size_t)t * nb + b] = run;
      run += v;
    }
    tot[b] = run;
    big = max(big, run);
  }
  __syncthreads();
  // bucket starts: exclusive scan of the totals (each thread a run of buckets)
  const int per = (nb + blockDim.x - 1) / blockDim.x;
  const int b0 = threadIdx.x * per;
  uint32_t sum = 0;
  for (int b = b0; b < min(b0 + per, nb); ++b) sum += tot[b];
  uint32_t run = block_exclusive_sum<1024>(sum, s_warp, &s_total) + (uint32_t)start[c];
  for (int b = b0; b < min(b0 + per, nb); ++b) {
    const uint32_t t = tot[b];
    bstart[(size_t)c * nb + b] = run;
    bcount[(size_t)c * nb + b] = t;
    tot[b] = run;
    run += t;
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int t = t0; t < t1; ++t) tile_off[(size_t)t * nb + b] += tot[b];
  big = __reduce_max_sync(0xffffffffu, big);
  if ((threadIdx.x & 31) == 0 && big) atomicMax(&stats->max_bucket, big);
}

__global__ void __launch_bounds__(256)
    lb_scatter_kernel(const uint32_t* __restrict__ keys, uint32_t* __restrict__ out,
                      const int4* __restrict__ tiles, int n_tiles, const char* __restrict__ blob,
                      LcdfLayout L, int nb, const uint32_t* __restrict__ tile_off) {
  extern __shared__ __align__(16) unsigned char sm[];
  uint32_t* cursor = reinterpret_cast<uint32_t*>(sm);
  const BucketLookup q =
      load_lookup(blob, L, nb, cursor + nb, reinterpret_cast<uint16_t*>(cursor + 2 * nb));
  const int lane = threadIdx.x & 31;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const uint32_t* row = tile_off + (size_t)t * nb;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) cursor[b] = row[b];
    __syncthreads();
    const int4 d = tiles[t];
    for (int base = d.x + (int)(threadIdx.x >> 5) * 32 * kLbRows; base < d.y;
         base += blockDim.x * kLbRows) {
      uint32_t k[kLbRows];
#pragma unroll
      for (int u = 0; u < kLbRows; ++u) {
        const int i = base + u * 32 + lane;
        k[u] = i < d.y ? keys[i] : 0xffffffffu;
      }
#pragma unroll
      for (int u = 0; u < kLbRows; ++u)
        if (lb_first_of_its_key(k[u])) out[atomicAdd(&cursor[bucket_of(q, k[u])], 1u)] = k[u];
    }
    __syncthreads();
  }
}

// Per cloud: unique-run offsets (absolute positions) and the cloud's U.
__global__ void __launch_bounds__(1024)
    lb_uscan_kernel(const int* __restrict__ start, int nb, const uint32_t* __restrict__ ucount,
                    uint32_t* __restrict__ uoff, uint32_t* __restrict__ ucloud,
                    const LsortStats* __restrict__ stats) {
  if (stats->fallback) return;
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  const int c = blockIdx.x;
  const int per = (nb + blockDim.x - 1) / blockDim.x;
  const int b0 = threadIdx.x * per;
  const uint32_t* uc = ucount + (size_t)c * nb;
  uint32_t sum = 0;
  for (int b = b0; b < min(b0 + per, nb); ++b) sum += uc[b];
  uint32_t run = block_exclusive_sum<1024>(sum, s_warp, &s_total) + (uint32_t)start[c];
  for (int b = b0; b < min(b0 + per, nb); ++b) {
    uoff[(size_t)c * nb + b] = run;
    run += uc[b];
  }
  if (threadIdx.x == 0) ucloud[c] = s_total;
}

__global__ void __launch_bounds__(256)
    lb_compact_kernel(const uint32_t* __restrict__ bkeys, const uint32_t* __restrict__ bstart,
                      const uint32_t* __restrict__ ucount, const uint32_t* __restrict__ uoff,
                      uint32_t* __restrict__ out, const LsortStats* __restrict__ stats) {
  if (stats->fallback) return;
  const int g = blockIdx.x;
  copy_run(out + uoff[g], bkeys + bstart[g], ucount[g]);
}

__global__ void __launch_bounds__(256)
    lb_pad_kernel(const int* __restrict__ start, const uint32_t* __restrict__ ucloud,
                  uint32_t* __restrict__ out, const LsortStats* __restrict__ stats) {
  if (stats->fallback) return;
  const int c = blockIdx.x;
  const int s0 = start[c], s1 = start[c + 1];
  const int u = (int)ucloud[c];
  if (u == 0) return;
  const uint32_t last = out[s0 + u - 1];
  for (int i = s0 + u + (int)threadIdx.x; i < s1; i += blockDim.x) out[i] = last;
}

size_t lbatch_scratch_bytes(int n_tiles, int n_clouds, int nb, int n) {
  const size_t g = (size_t)n_clouds * nb;
  return align_up(4 * (size_t)n_tiles * nb, 256) + 4 * align_up(4 * g, 256) +
         align_up(4 * (size_t)n_clouds, 256) +
         align_up(4 * (size_t)(n > 0 ? n : 1), 256);
}

cudaError_t launch_lbatch_sort(const LbatchArgs& a, cudaStream_t s) {
  if (a.n_tiles <= 0) return cudaSuccess;
  const size_t G = (size_t)a.C * a.nb;
  char* w = static_cast<char*>(a.scratch);
  auto take = [&](size_t bytes) {
    char* p = w;
    w += align_up(bytes, 256);
    return reinterpret_cast<uint32_t*>(p);
  };
  uint32_t* tile_off = take(4 * (size_t)a.n_tiles * a.nb);
  uint32_t* bstart = take(4 * G);
  uint32_t* bcount = take(4 * G);
  uint32_t* ucount = take(4 * G);
  uint32_t* uoff = take(4 * G);
  uint32_t* ucloud = take(4 * (size_t)a.C);
  uint32_t* bkeys = take(4 * (size_t)(a.n > 0 ? a.n : 1));
  const size_t hsm = lsort_hist_smem(a.nb, a.L.max_knots);
  if (hsm > (size_t)kLsortMaxSmem) return cudaErrorInvalidValue;
  cudaError_t e = set_smem_limit(lb_hist_kernel, (int)hsm);
  if (e == cudaSuccess) e = set_smem_limit(lb_scatter_kernel, (int)hsm);
  if (e == cudaSuccess) e = set_smem_limit(lsort_bucket_kernel, (int)sizeof(BucketSmem));
  if (e != cudaSuccess) return e;
  const int tgrid = std::min(a.n_tiles, device_sm_count() * 6);
  lb_hist_kernel<<<tgrid, 256, hsm, s>>>(a.keys, a.tiles, a.n_tiles, a.blob, a.L, a.nb, tile_off);
  lb_scan_kernel<<<a.C, 1024, 4 * (size_t)a.nb, s>>>(a.start, a.cloud_tile0, a.nb, a.C, tile_off,
                                                     bstart, bcount, a.stats);
  lb_scatter_kernel<<<tgrid, 256, hsm, s>>>(a.keys, bkeys, a.tiles, a.n_tiles, a.blob, a.L, a.nb,
                                            tile_off);
  lsort_bucket_kernel<<<(unsigned)G, kBkThreads, sizeof(BucketSmem), s>>>(bkeys, bstart, ucount,
                                                                          a.stats, bcount);
  lb_uscan_kernel<<<a.C, 1024, 0, s>>>(a.start, a.nb, ucount, uoff, ucloud, a.stats);
  lb_compact_kernel<<<(unsigned)G, 256, 0, s>>>(bkeys, bstart, ucount, uoff, a.out, a.stats);
  lb_pad_kernel<<<a.C, 256, 0, s>>>(a.start, ucloud, a.out, a.stats);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ plan --
LsortPlan lsort_plan(int n, int nb, int max_segments) {
  LsortPlan p{};
  p.n = n;
  p.nb = nb;
  p.L = lcdf_layout(max_segments);
  p.fallback_sort = sort_plan(n, 30);
  p.fallback_unique = unique_plan(n);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o = align_up(o + bytes, 256);
    return at;
  };
  // zeroed each run: everything up to the end of the fallback sort's zeroed
  // part (its bases and per-tile histograms follow, written before use)
  p.stats_off = take(sizeof(LsortStats));
  p.cursor_off = take(4 * (size_t)nb);
  p.uniq_ctrl_off = take(p.fallback_unique.bytes);
  p.sort_ctrl_off = take(p.fallback_sort.bytes);
  p.zero_bytes = p.sort_ctrl_off + p.fallback_sort.zero_bytes;
  // not zeroed:
  p.starts_off = take(4 * (size_t)(nb + 1));
  p.ucount_off = take(4 * (size_t)nb);
  p.uoff_off = take(4 * (size_t)nb);
  p.counts_off = take(4 * (size_t)nb);
  // bucket capacity of the one-pass bin (a bucket past it sends the sort to
  // the fallback): what the bucket kernel's sorted forms take (kCap keys;
  // only a bitmap takes more), or 2x the mean bucket when that is larger; a
  // whole number of 128-byte lines
  const size_t mean = ((size_t)(n > 0 ? n : 1) + nb - 1) / nb;
  p.cap = (uint32_t)align_up(std::max<size_t>((size_t)kCap, 2 * mean), 32);
  p.bkeys_off = take(4 * (size_t)nb * p.cap);
  p.alt_off = take(4 * (size_t)(n > 0 ? n : 1));
  p.bytes = o;
  return p;
}

cudaError_t launch_lsort(const float4* pts, uint32_t* keys, int n, float min_coord, float range,
                         const char* blob, const LsortPlan& p, char* ws, float threshold,
                         uint32_t* out, int* d_unique, uint32_t* status, cudaStream_t s,
                         Recorder* rec) {
  if (n <= 0) return cudaMemsetAsync(d_unique, 0, sizeof(int), s);
  LsortStats* stats = reinterpret_cast<LsortStats*>(ws + p.stats_off);
  // the fallback launches run only when the learned path gave up: their gate
  // is the fallback flag itself (final once the bucket kernel is done)
  uint32_t* gate = &stats->fallback;
  uint32_t* starts = reinterpret_cast<uint32_t*>(ws + p.starts_off);
  uint32_t* ucount = reinterpret_cast<uint32_t*>(ws + p.ucount_off);
  uint32_t* uoff = reinterpret_cast<uint32_t*>(ws + p.uoff_off);
  uint32_t* bkeys = reinterpret_cast<uint32_t*>(ws + p.bkeys_off);
  uint32_t* alt = reinterpret_cast<uint32_t*>(ws + p.alt_off);
  uint32_t* cursor = reinterpret_cast<uint32_t*>(ws + p.cursor_off);
  uint32_t* counts = reinterpret_cast<uint32_t*>(ws + p.counts_off);
  const size_t bsm = lsort_bin_smem(p.nb);
  if (bsm > (size_t)kLsortMaxSmem) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(lsort_bin_kernel<true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsm);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(lsort_bin_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bsm);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(lsort_bucket_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(BucketSmem));
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(ws, 0, p.zero_bytes, s);
  if (e != cudaSuccess) return e;
  mark(rec, s);
  // kBinCtasPerSm CTAs per SM, each taking the same number of tiles (rounds)
  // of at most kBinTile keys: small clouds spread over every SM, large ones
  // leave no partial last round
  const int sms = device_sm_count() * kBinCtasPerSm;
  const long long per_round = (long long)sms * kBinTile;
  const int rounds = (int)std::max(1LL, ((long long)n + per_round - 1) / per_round);
  const long long slots = (long long)sms * rounds;
  const int tile = (int)std::max(1LL, ((long long)n + slots - 1) / slots);
  const int tiles = (n + tile - 1) / tile;
  const int grid = std::min(sms, tiles);
  if (pts)
    lsort_bin_kernel<true><<<grid, kBinThreads, bsm, s>>>(pts, keys, n, min_coord, range, blob, p.L,
                                                          p.nb, p.cap, tile, cursor, bkeys,
                                                          status);
  else
    lsort_bin_kernel<false><<<grid, kBinThreads, bsm, s>>>(nullptr, keys, n, 0.f, 1.f, blob, p.L,
                                                           p.nb, p.cap, tile, cursor, bkeys,
                                                           status);
  mark(rec, s);
  lsort_bin_stats_kernel<<<1, 1024, 0, s>>>(cursor, p.nb, n, p.cap, threshold, blob, starts, counts,
                                            stats);
  mark(rec, s);
  lsort_bucket_kernel<<<p.nb, kBkThreads, sizeof(BucketSmem), s>>>(bkeys, starts, ucount, stats,
                                                                   counts);
  mark(rec, s);
  lsort_uscan_kernel<<<1, 1024, 0, s>>>(ucount, p.nb, uoff, d_unique, stats);
  lsort_compact_kernel<<<p.nb, 256, 0, s>>>(bkeys, starts, ucount, uoff, out, stats);
  mark(rec, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // Fallback: OneSweep + unique on the original keys, gated on the flag.
  char* sc = ws + p.sort_ctrl_off;
  e = launch_histogram_gated(keys, &p.fallback_sort, sc, gate, s);
  if (e != cudaSuccess) return e;
  uint32_t* sorted = keys;
  e = launch_sort_passes_gated(keys, alt, &p.fallback_sort, sc, status, gate, s, &sorted);
  if (e != cudaSuccess) return e;
  e = launch_unique_gated(sorted, out, n, d_unique, &p.fallback_unique, ws + p.uniq_ctrl_off,
                          status, gate, s);
  mark(rec, s);
  return e;
}

}  // namespace octgb

// ------------------------------------------------------------------ C ABI --
namespace {

struct LearnedBuildLayout {
  octgb::LsortPlan lp;
  size_t misc_off, lsort_off, keys_off, tree_off, tags_off, total;
};

LearnedBuildLayout learned_layout(int n, int cap, int nb, int max_segments) {
  using namespace octgb;
  LearnedBuildLayout L{};
  L.lp = lsort_plan(n, nb, max_segments);
  L.misc_off = 0;
  L.lsort_off = 256;
  L.keys_off = align_up(L.lsort_off + L.lp.bytes, 256);
  L.tree_off = align_up(L.keys_off + 4 * (size_t)(n > 0 ? n : 1), 256);
  L.tags_off = align_up(L.tree_off + tree_scratch_bytes(n), 256);
  L.total = align_up(L.tags_off + oct_tags_bytes(cap), 256);
  return L;
}

bool lsort_args_ok(int n, int nb, int max_segments) {
  return n >= 0 && n <= OCT_MAX_N && nb >= 1 && nb <= 65536 && max_segments >= 1 &&
         max_segments <= octgb::kLcdfMaxSegments &&
         octgb::lsort_hist_smem(nb, max_segments) <= (size_t)octgb::kLsortMaxSmem &&
         octgb::lsort_bin_smem(nb) <= (size_t)octgb::kLsortMaxSmem;
}

int fail_cuda(cudaError_t e, const char* where) {
  char msg[192];
  snprintf(msg, sizeof(msg), "%s: %s", where, cudaGetErrorString(e));
  octgb::set_last_error(msg);
  return OCT_ERR_CUDA;
}

}  // namespace

extern "C" {

OCT_API int oct_set_sort_config(int radix_bits, int warps, int items, int scan) {
  using namespace octgb;
  const SortConfig c{radix_bits, warps, items, scan};
  const SortPlan p = sort_plan_cfg(1 << 20, 30, c);
  if (p.cfg.radix_bits != radix_bits || p.cfg.items != items || p.cfg.scan != scan)
    return OCT_ERR_INVALID_ARG;
  set_sort_config(c);
  return OCT_OK;
}

OCT_API int oct_get_sort_config(int out[4]) {
  if (!out) return OCT_ERR_INVALID_ARG;
  const octgb::SortConfig c = octgb::get_sort_config();
  out[0] = c.radix_bits;
  out[1] = c.warps;
  out[2] = c.items;
  out[3] = c.scan;
  return OCT_OK;
}

OCT_API size_t oct_lsort_workspace_bytes(int n, int n_buckets, int max_segments) {
  if (!lsort_args_ok(n, n_buckets, max_segments)) return 0;
  return octgb::lsort_plan(n, n_buckets, max_segments).bytes;
}

OCT_API int oct_lsort_unique(uint32_t* keys, int n, const void* model, int max_segments,
                             int n_buckets, float overflow_threshold, uint32_t* out_unique,
                             int32_t* d_n_unique, void* d_stats, void* workspace,
                             size_t workspace_bytes, uint32_t* d_status, oct_stream_t stream) {
  using namespace octgb;
  if (!lsort_args_ok(n, n_buckets, max_segments) || !model || !d_n_unique ||
      (n > 0 && (!keys || !out_unique || !workspace)) ||
      (reinterpret_cast<uintptr_t>(workspace) & 255))
    return OCT_ERR_INVALID_ARG;
  const LsortPlan p = lsort_plan(n, n_buckets, max_segments);
  if (n > 0 && workspace_bytes < p.bytes) return OCT_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  cudaError_t e = launch_lsort(nullptr, keys, n, 0.f, 1.f, static_cast<const char*>(model), p, ws,
                               overflow_threshold, out_unique, d_n_unique, d_status, s, nullptr);
  if (e == cudaSuccess && d_stats && n > 0)
    e = cudaMemcpyAsync(d_stats, ws + p.stats_off, sizeof(LsortStats), cudaMemcpyDeviceToDevice, s);
  return e == cudaSuccess ? OCT_OK : fail_cuda(e, "oct_lsort_unique");
}

OCT_API size_t oct_build_learned_workspace_bytes(int n, int nodes_capacity, int n_buckets,
                                                 int max_segments) {
  if (!lsort_args_ok(n, n_buckets, max_segments) || nodes_capacity < 0) return 0;
  return learned_layout(n, nodes_capacity, n_buckets, max_segments).total;
}

OCT_API int oct_build_octree_learned(const oct_vec4* points, int n, float min_coord, float range,
                                     const void* model, int max_segments, int n_buckets,
                                     float overflow_threshold, const oct_build_outputs* out,
                                     void* d_stats, void* workspace, size_t workspace_bytes,
                                     oct_stream_t stream) {
  using namespace octgb;
  if (!lsort_args_ok(n, n_buckets, max_segments) || !model || !out || !out->d_counts)
    return OCT_ERR_INVALID_ARG;
  if (out->nodes_capacity > 0 && n > OCT_MAX_OCTREE_NODES + 1) return OCT_ERR_TOO_LARGE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (n == 0) {
    const cudaError_t e = cudaMemsetAsync(out->d_counts, 0, 4 * sizeof(int32_t), s);
    return e == cudaSuccess ? OCT_OK : fail_cuda(e, "oct_build_octree_learned");
  }
  if (!points || (reinterpret_cast<uintptr_t>(points) & 15) || !out->codes ||
      !out->tree.prefix_n || !out->tree.has_leaf_left || !out->tree.has_leaf_right ||
      !out->tree.left_child || !out->tree.parent || !out->edge_count || !out->prefix_sum ||
      out->nodes_capacity < 0 || (out->nodes_capacity > 0 && !out->nodes) || !workspace ||
      (reinterpret_cast<uintptr_t>(workspace) & 255))
    return OCT_ERR_INVALID_ARG;
  const LearnedBuildLayout L = learned_layout(n, out->nodes_capacity, n_buckets, max_segments);
  if (workspace_bytes < L.total) return OCT_ERR_WORKSPACE;
  char* w = static_cast<char*>(workspace);
  uint32_t* status = reinterpret_cast<uint32_t*>(w + L.misc_off);
  int* d_unique = reinterpret_cast<int*>(w + L.misc_off + 4);
  int* d_max_slot = reinterpret_cast<int*>(w + L.misc_off + 8);
  uint32_t* keys = reinterpret_cast<uint32_t*>(w + L.keys_off);
  cudaError_t e = cudaMemsetAsync(w, 0, L.lsort_off, s);  // misc
  if (e == cudaSuccess)
    e = launch_lsort(reinterpret_cast<const float4*>(points), keys, n, min_coord, range,
                     static_cast<const char*>(model), L.lp, w + L.lsort_off, overflow_threshold,
                     out->codes, d_unique, status, s, nullptr);
  if (e == cudaSuccess)
    e = launch_radix_tree_sorted(n, d_unique, out->codes, out->tree.prefix_n,
                                 out->tree.has_leaf_left, out->tree.has_leaf_right,
                                 out->tree.left_child, out->tree.parent, out->edge_count,
                                 w + L.tree_off, s);
  const OctTags tags = oct_tags_carve(w + L.tags_off, out->nodes_capacity);
  if (e == cudaSuccess)
    e = launch_prefix_sum_clear_tags(n, d_unique, out->edge_count, out->prefix_sum, d_max_slot,
                                     w + L.tree_off, status, tags, s);
  if (e == cudaSuccess && out->nodes_capacity > 0) {
    OctArgs a{};
    a.nodes = out->nodes;
    a.cap = out->nodes_capacity;
    a.offsets = out->prefix_sum;
    a.counts = out->edge_count;
    a.codes = out->codes;
    a.prefix_n = out->tree.prefix_n;
    a.hll = out->tree.has_leaf_left;
    a.hlr = out->tree.has_leaf_right;
    a.parent = out->tree.parent;
    a.left_child = out->tree.left_child;
    a.min_coord = min_coord;
    a.range = range;
    a.n_brt_host = n;
    a.d_unique = d_unique;
    a.d_max_slot = d_max_slot;
    e = launch_octree(kOctMake | kOctLink | kOctFresh, a, tags, status, s, nullptr, true);
  }
  if (e == cudaSuccess) e = launch_publish_counts(d_unique, d_max_slot, status, out->d_counts, s);
  if (e == cudaSuccess && d_stats)
    e = cudaMemcpyAsync(d_stats, w + L.lsort_off + L.lp.stats_off, sizeof(LsortStats),
                        cudaMemcpyDeviceToDevice, s);
  return e == cudaSuccess ? OCT_OK : fail_cuda(e, "oct_build_octree_learned");
}

}  // extern "C"
