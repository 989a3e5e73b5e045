// Learned bucketed sort + unique (stages 2-3 driven by the learned CDF).
//
// With a model whose bucket(v) never decreases with v, sorting reduces to a
// scatter into buckets followed by an independent sort of each bucket, and the
// unique pass fuses into the bucket stage (equal keys share a bucket):
//
//   hist     per-chunk bucket counts (Morton fused when starting from points)
//   offsets  per-bucket totals and per-chunk offsets; bucket starts; overflow
//            fraction (keys in buckets above the shared-memory capacity) and
//            the fallback decision when it exceeds the threshold
//   scatter  each chunk writes its keys into its reserved bucket ranges
//   buckets  one CTA per bucket: the sorted unique keys of the bucket from a
//            shared-memory bitmap over [min, max] of its keys when that span
//            fits (any key count), else a bitonic sort of the keys in shared
//            memory (up to kCap keys); decoupled look-back across buckets
//            gives each bucket's output offset.
//
// If any bucket fits neither form, or the overflow fraction exceeds the
// threshold, the device flag `fallback` is set and the OneSweep sort + unique
// (launched right after, gated on the flag) redo stages 2-3 from the original
// keys; otherwise those launches return at once. Either way the output is the
// sorted unique key array, identical to the plain path's.
#include <stdio.h>

#include "learned.cuh"
#include "lsort.cuh"

namespace octgb {

constexpr int kBmBits = 1 << 19;          // bitmap span limit (64 KiB of shared memory)
constexpr int kBmWords = kBmBits / 32;
constexpr int kCap = 16384;               // bitonic-sort capacity (keys; the 64 KiB buffer)
constexpr int kBucketThreads = 512;

// ------------------------------------------------------------- histogram --
template <bool FROM_POINTS>
__global__ void __launch_bounds__(256)
    lsort_hist_kernel(const float4* __restrict__ pts, uint32_t* __restrict__ keys, int n,
                      float min_coord, float range, const char* __restrict__ blob, LcdfLayout L,
                      uint32_t* __restrict__ chunk_hist, int nb, uint32_t* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char sm[];
  uint32_t* s_hist = reinterpret_cast<uint32_t*>(sm);
  LcdfTables t = lcdf_load_tables(blob, L, sm + align_up(4 * (size_t)nb, 16));
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s_hist[b] = 0;
  __syncthreads();
  const int G = gridDim.x, c = blockIdx.x;
  const int lo = (int)((long long)n * c / G), hi = (int)((long long)n * (c + 1) / G);
  bool bad = false;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    uint32_t code;
    if (FROM_POINTS) {
      const float4 p = ld_stream_f4(pts + i);
      bad |= !(in_range(p.x, min_coord, range) && in_range(p.y, min_coord, range) &&
               in_range(p.z, min_coord, range));
      code = morton_code(p.x, p.y, p.z, min_coord, range);
      keys[i] = code;
    } else {
      code = keys[i];
    }
    atomicAdd(&s_hist[min(lcdf_bucket(t, code), (uint32_t)(nb - 1))], 1u);
  }
  if (FROM_POINTS && __syncthreads_or(bad) && threadIdx.x == 0) raise_status(status, kStatusRange);
  __syncthreads();
  uint32_t* row = chunk_hist + (size_t)c * nb;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) row[b] = s_hist[b];
}

// --------------------------------------------------------------- offsets --
// Block: 32 buckets x 8 chunk groups. chunk_hist[c][b] becomes the exclusive
// offset of chunk c inside bucket b; totals[b] the bucket's count.
__global__ void __launch_bounds__(256)
    lsort_offsets_kernel(uint32_t* __restrict__ chunk_hist, int G, int nb,
                         uint32_t* __restrict__ totals) {
  __shared__ uint32_t part[8][33];
  const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int b = blockIdx.x * 32 + l;
  const int c0 = (int)((long long)G * w / 8), c1 = (int)((long long)G * (w + 1) / 8);
  uint32_t sum = 0;
  if (b < nb)
    for (int c = c0; c < c1; ++c) sum += chunk_hist[(size_t)c * nb + b];
  part[w][l] = sum;
  __syncthreads();
  uint32_t base = 0;
  for (int k = 0; k < w; ++k) base += part[k][l];
  if (w == 7 && b < nb) totals[b] = base + sum;
  if (b < nb) {
    uint32_t run = base;
    for (int c = c0; c < c1; ++c) {
      const uint32_t v = chunk_hist[(size_t)c * nb + b];
      chunk_hist[(size_t)c * nb + b] = run;
      run += v;
    }
  }
}

// One block: bucket starts (exclusive scan of totals), overflow fraction and
// the fallback decision.
__global__ void __launch_bounds__(1024)
    lsort_scan_kernel(const uint32_t* __restrict__ totals, int nb, int n, float threshold,
                      uint32_t* __restrict__ starts, LsortStats* __restrict__ stats) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t total;
  __shared__ uint32_t s_over, s_max;
  if (threadIdx.x == 0) {
    s_over = 0;
    s_max = 0;
  }
  __syncthreads();
  const int per = (nb + 1023) / 1024;
  uint32_t sum = 0, over = 0, mx = 0;
  for (int j = 0; j < per; ++j) {
    const int b = threadIdx.x * per + j;
    if (b < nb) {
      const uint32_t v = totals[b];
      sum += v;
      if (v > (uint32_t)kCap) over += v;
      mx = max(mx, v);
    }
  }
  atomicAdd(&s_over, over);
  atomicMax(&s_max, mx);
  uint32_t run = block_exclusive_sum<1024>(sum, warp_tot, &total);
  for (int j = 0; j < per; ++j) {
    const int b = threadIdx.x * per + j;
    if (b < nb) {
      starts[b] = run;
      run += totals[b];
    }
  }
  if (threadIdx.x == 0) {
    starts[nb] = total;
    stats->overflow_keys = s_over;
    stats->max_bucket = s_max;
    stats->n = (uint32_t)n;
    const float frac = n > 0 ? (float)s_over / (float)n : 0.f;
    stats->overflow_frac = frac;
    // Fallback when too many keys sit in oversized buckets (load imbalance).
    if (frac > threshold) {
      stats->skip = 1u;
      stats->fallback = 1u;
    }
  }
}

// --------------------------------------------------------------- scatter --
__global__ void __launch_bounds__(256)
    lsort_scatter_kernel(const uint32_t* __restrict__ keys, int n, const char* __restrict__ blob,
                         LcdfLayout L, const uint32_t* __restrict__ chunk_off,
                         const uint32_t* __restrict__ starts, int nb, uint32_t* __restrict__ out,
                         const LsortStats* __restrict__ stats) {
  if (stats->skip) return;
  extern __shared__ __align__(16) unsigned char sm[];
  uint32_t* cursor = reinterpret_cast<uint32_t*>(sm);
  LcdfTables t = lcdf_load_tables(blob, L, sm + align_up(4 * (size_t)nb, 16));
  const int G = gridDim.x, c = blockIdx.x;
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    cursor[b] = starts[b] + chunk_off[(size_t)c * nb + b];
  __syncthreads();
  const int lo = (int)((long long)n * c / G), hi = (int)((long long)n * (c + 1) / G);
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const uint32_t k = keys[i];
    const uint32_t pos = atomicAdd(&cursor[min(lcdf_bucket(t, k), (uint32_t)(nb - 1))], 1u);
    if (pos < (uint32_t)n) out[pos] = k;
  }
}

// ---------------------------------------------------------------- buckets --
constexpr unsigned long long kLbAggB = 1ull << 62;
constexpr unsigned long long kLbIncB = 2ull << 62;
constexpr unsigned long long kLbFlagsB = 3ull << 62;

__device__ uint32_t bucket_lookback(unsigned long long* lb, int tile, uint32_t agg,
                                    uint32_t* status) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) st_release_u64(lb, kLbIncB | agg);
    return 0;
  }
  if (lane == 0) st_release_u64(lb + tile, kLbAggB | agg);
  uint32_t ex = 0;
  int pred = tile - 1;
  uint32_t spins = 0;
  while (true) {
    const int p = pred - lane;
    const unsigned long long w = p >= 0 ? ld_relaxed_u64(lb + p) : kLbIncB;
    const unsigned long long f = w & kLbFlagsB;
    const uint32_t inc_m = __ballot_sync(0xffffffffu, f == kLbIncB);
    const uint32_t nr_m = __ballot_sync(0xffffffffu, f == 0);
    const int first_inc = inc_m ? __ffs(inc_m) - 1 : 32;
    const int first_nr = nr_m ? __ffs(nr_m) - 1 : 32;
    if (first_nr < first_inc) {
      ex += __reduce_add_sync(0xffffffffu, lane < first_nr ? (uint32_t)w : 0u);
      pred -= first_nr;
      if (++spins > kSpinLimit) {
        if (lane == 0) raise_status(status, kStatusSpinTimeout);
        break;
      }
      backoff(spins);
      continue;
    }
    const int take = first_inc < 32 ? first_inc + 1 : 32;
    ex += __reduce_add_sync(0xffffffffu, lane < take ? (uint32_t)w : 0u);
    if (first_inc < 32) break;
    pred -= 32;
  }
  if (lane == 0) st_release_u64(lb + tile, kLbIncB | (uint32_t)(ex + agg));
  return ex;
}

struct BucketSmem {
  uint32_t bitmap[kBmWords];  // 64 KiB; the bitonic path reuses it for keys
  uint32_t warp_tot[32];
  uint32_t misc[8];
};

__global__ void __launch_bounds__(kBucketThreads)
    lsort_bucket_kernel(const uint32_t* __restrict__ bkeys, const uint32_t* __restrict__ starts,
                        int nb, uint32_t* __restrict__ out, int* __restrict__ d_unique,
                        unsigned long long* __restrict__ lb, uint32_t* __restrict__ counter,
                        LsortStats* __restrict__ stats, uint32_t* __restrict__ status) {
  // `skip` is final before this kernel starts; `fallback` may still be set by
  // a failing bucket, and every bucket must publish its count regardless.
  if (stats->skip) return;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  BucketSmem& S = *reinterpret_cast<BucketSmem*>(sm_raw);
  const int tid = threadIdx.x;
  if (tid == 0) S.misc[0] = atomicAdd(counter, 1u);
  __syncthreads();
  const int b = (int)S.misc[0];
  const uint32_t lo = starts[b], hi = starts[b + 1];
  const int cnt = (int)(hi - lo);
  // key span of the bucket
  uint32_t kmin = 0xffffffffu, kmax = 0;
  for (int i = tid; i < cnt; i += kBucketThreads) {
    const uint32_t k = bkeys[lo + i];
    kmin = min(kmin, k);
    kmax = max(kmax, k);
  }
  kmin = __reduce_min_sync(0xffffffffu, kmin);
  kmax = __reduce_max_sync(0xffffffffu, kmax);
  if ((tid & 31) == 0) {
    S.warp_tot[tid >> 5] = kmin;
  }
  __syncthreads();
  if (tid < 32) {
    uint32_t v = tid < kBucketThreads / 32 ? S.warp_tot[tid] : 0xffffffffu;
    v = __reduce_min_sync(0xffffffffu, v);
    if (tid == 0) S.misc[1] = v;
  }
  __syncthreads();
  if ((tid & 31) == 0) S.warp_tot[tid >> 5] = kmax;
  __syncthreads();
  if (tid < 32) {
    uint32_t v = tid < kBucketThreads / 32 ? S.warp_tot[tid] : 0u;
    v = __reduce_max_sync(0xffffffffu, v);
    if (tid == 0) S.misc[2] = v;
  }
  __syncthreads();
  kmin = S.misc[1];
  kmax = S.misc[2];
  const uint32_t span = cnt > 0 ? kmax - kmin + 1u : 0u;

  uint32_t uniq = 0;
  int path;  // 0 bitmap, 1 bitonic, 2 cannot
  if (cnt == 0) path = 0;
  else if (span <= (uint32_t)kBmBits) path = 0;
  else if (cnt <= kCap) path = 1;
  else path = 2;

  if (path == 2) {
    if (tid == 0) {
      atomicOr(&stats->fallback, 1u);
      atomicAdd(&stats->failed_buckets, 1u);
    }
    // still publish a count so later buckets' look-backs end
  }

  const int words = path == 0 ? (int)((span + 31) >> 5) : 0;
  if (path == 0 && cnt > 0) {
    for (int w = tid; w < words; w += kBucketThreads) S.bitmap[w] = 0;
    __syncthreads();
    for (int i = tid; i < cnt; i += kBucketThreads) {
      const uint32_t r = bkeys[lo + i] - kmin;
      atomicOr(&S.bitmap[r >> 5], 1u << (r & 31));
    }
    __syncthreads();
  } else if (path == 1) {
    // bitonic sort of cnt keys padded to a power of two with 0xffffffff
    int m = 1;
    while (m < cnt) m <<= 1;
    for (int i = tid; i < m; i += kBucketThreads) S.bitmap[i] = i < cnt ? bkeys[lo + i] : 0xffffffffu;
    __syncthreads();
    for (int k = 2; k <= m; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = tid; i < m; i += kBucketThreads) {
          const int p = i ^ j;
          if (p > i) {
            const uint32_t a = S.bitmap[i], c = S.bitmap[p];
            const bool up = (i & k) == 0;
            if ((a > c) == up) {
              S.bitmap[i] = c;
              S.bitmap[p] = a;
            }
          }
        }
        __syncthreads();
      }
    }
  }

  // Count unique keys: bitmap popcounts, or run heads of the sorted keys.
  constexpr int kPer = kBmWords / kBucketThreads;  // words per thread (contiguous)
  uint32_t mine = 0;
  if (path == 0) {
    const int w0 = tid * kPer;
#pragma unroll 4
    for (int q = 0; q < kPer; ++q)
      if (w0 + q < words) mine += __popc(S.bitmap[w0 + q]);
  } else if (path == 1) {
    const int per = (cnt + kBucketThreads - 1) / kBucketThreads;
    const int i0 = tid * per;
    for (int q = 0; q < per; ++q) {
      const int i = i0 + q;
      if (i < cnt && (i == 0 || S.bitmap[i] != S.bitmap[i - 1])) ++mine;
    }
  }
  uint32_t total_u;
  const uint32_t my_off = block_exclusive_sum<kBucketThreads>(mine, S.warp_tot, &S.misc[3]);
  total_u = S.misc[3];
  uniq = path == 2 ? 0u : total_u;
  if (tid < 32) {
    const uint32_t e = bucket_lookback(lb, b, uniq, status);
    if (tid == 0) S.misc[4] = e;
  }
  __syncthreads();
  const uint32_t ex = S.misc[4];
  if (path == 0 && cnt > 0) {
    uint32_t o = ex + my_off;
    const int w0 = tid * kPer;
    for (int q = 0; q < kPer; ++q) {
      const int w = w0 + q;
      if (w >= words) break;
      uint32_t bits = S.bitmap[w];
      while (bits) {
        const int bit = __ffs(bits) - 1;
        bits &= bits - 1;
        out[o++] = kmin + ((uint32_t)w << 5) + (uint32_t)bit;
      }
    }
  } else if (path == 1) {
    const int per = (cnt + kBucketThreads - 1) / kBucketThreads;
    const int i0 = tid * per;
    uint32_t o = ex + my_off;
    for (int q = 0; q < per; ++q) {
      const int i = i0 + q;
      if (i < cnt && (i == 0 || S.bitmap[i] != S.bitmap[i - 1])) out[o++] = S.bitmap[i];
    }
  }
  if (tid == 0 && b == nb - 1) *d_unique = (int)(ex + uniq);
}

// Gate for the fallback launches: 1 when the learned path gave up.
__global__ void lsort_gate_kernel(const LsortStats* stats, uint32_t* gate) {
  *gate = stats->fallback ? 1u : 0u;
}

// ------------------------------------------------------------------ plan --
LsortPlan lsort_plan(int n, int nb, int max_segments) {
  LsortPlan p{};
  p.n = n;
  p.nb = nb;
  p.chunks = device_sm_count() * 2;
  p.L = lcdf_layout(max_segments);
  p.fallback_sort = sort_plan(n, 30);
  p.fallback_unique = unique_plan(n);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o = align_up(o + bytes, 256);
    return at;
  };
  // zeroed each run:
  p.stats_off = take(sizeof(LsortStats));
  p.counter_off = take(64);
  p.lookback_off = take(8 * (size_t)(nb + 1));
  p.sort_ctrl_off = take(p.fallback_sort.bytes);
  p.uniq_ctrl_off = take(p.fallback_unique.bytes);
  p.zero_bytes = o;
  // not zeroed:
  p.hist_off = take(4 * (size_t)p.chunks * nb);
  p.totals_off = take(4 * (size_t)nb);
  p.starts_off = take(4 * (size_t)(nb + 1));
  p.bkeys_off = take(4 * (size_t)(n > 0 ? n : 1));
  p.alt_off = take(4 * (size_t)(n > 0 ? n : 1));
  p.bytes = o;
  return p;
}

size_t lsort_hist_smem(int nb, int max_segments) {
  return align_up(4 * (size_t)nb, 16) + lcdf_tables_smem(max_segments);
}

cudaError_t launch_lsort(const float4* pts, uint32_t* keys, int n, float min_coord, float range,
                         const char* blob, const LsortPlan& p, char* ws, float threshold,
                         uint32_t* out, int* d_unique, uint32_t* status, cudaStream_t s,
                         Recorder* rec) {
  if (n <= 0) return cudaMemsetAsync(d_unique, 0, sizeof(int), s);
  LsortStats* stats = reinterpret_cast<LsortStats*>(ws + p.stats_off);
  uint32_t* counter = reinterpret_cast<uint32_t*>(ws + p.counter_off);
  uint32_t* gate = counter + 1;
  unsigned long long* lb = reinterpret_cast<unsigned long long*>(ws + p.lookback_off);
  uint32_t* hist = reinterpret_cast<uint32_t*>(ws + p.hist_off);
  uint32_t* totals = reinterpret_cast<uint32_t*>(ws + p.totals_off);
  uint32_t* starts = reinterpret_cast<uint32_t*>(ws + p.starts_off);
  uint32_t* bkeys = reinterpret_cast<uint32_t*>(ws + p.bkeys_off);
  uint32_t* alt = reinterpret_cast<uint32_t*>(ws + p.alt_off);
  const size_t hsm = lsort_hist_smem(p.nb, p.L.max_knots);
  if (hsm > (size_t)kLsortMaxSmem) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(lsort_hist_kernel<true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsm);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(lsort_hist_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hsm);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(lsort_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hsm);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(lsort_bucket_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(BucketSmem));
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(ws, 0, p.zero_bytes, s);
  if (e != cudaSuccess) return e;
  mark(rec, s);
  if (pts)
    lsort_hist_kernel<true><<<p.chunks, 256, hsm, s>>>(pts, keys, n, min_coord, range, blob, p.L,
                                                       hist, p.nb, status);
  else
    lsort_hist_kernel<false><<<p.chunks, 256, hsm, s>>>(nullptr, keys, n, 0.f, 1.f, blob, p.L,
                                                        hist, p.nb, status);
  mark(rec, s);
  lsort_offsets_kernel<<<(p.nb + 31) / 32, 256, 0, s>>>(hist, p.chunks, p.nb, totals);
  lsort_scan_kernel<<<1, 1024, 0, s>>>(totals, p.nb, n, threshold, starts, stats);
  mark(rec, s);
  lsort_scatter_kernel<<<p.chunks, 256, hsm, s>>>(keys, n, blob, p.L, hist, starts, p.nb, bkeys,
                                                  stats);
  mark(rec, s);
  lsort_bucket_kernel<<<p.nb, kBucketThreads, sizeof(BucketSmem), s>>>(
      bkeys, starts, p.nb, out, d_unique, lb, counter, stats, status);
  mark(rec, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // Fallback: OneSweep + unique on the original keys, gated on the flag.
  lsort_gate_kernel<<<1, 1, 0, s>>>(stats, gate);
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
  octgb::ScanPlan scan;
  size_t misc_off, scan_off, lsort_off, keys_off, tags_off, total;
};

LearnedBuildLayout learned_layout(int n, int cap, int nb, int max_segments) {
  using namespace octgb;
  LearnedBuildLayout L{};
  L.lp = lsort_plan(n, nb, max_segments);
  L.scan = edge_scan_plan(n);
  L.misc_off = 0;
  L.scan_off = 256;
  L.lsort_off = align_up(L.scan_off + L.scan.bytes, 256);
  L.keys_off = align_up(L.lsort_off + L.lp.bytes, 256);
  L.tags_off = align_up(L.keys_off + 4 * (size_t)(n > 0 ? n : 1), 256);
  L.total = align_up(L.tags_off + oct_tags_bytes(cap), 256);
  return L;
}

bool lsort_args_ok(int n, int nb, int max_segments) {
  return n >= 0 && n <= OCT_MAX_N && nb >= 1 && nb <= 65536 && max_segments >= 1 &&
         max_segments <= octgb::kLcdfMaxSegments &&
         octgb::lsort_hist_smem(nb, max_segments) <= (size_t)octgb::kLsortMaxSmem;
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
  cudaError_t e = cudaMemsetAsync(w, 0, L.lsort_off, s);  // misc + scan control
  if (e == cudaSuccess)
    e = launch_lsort(reinterpret_cast<const float4*>(points), keys, n, min_coord, range,
                     static_cast<const char*>(model), L.lp, w + L.lsort_off, overflow_threshold,
                     out->codes, d_unique, status, s, nullptr);
  if (e == cudaSuccess)
    e = launch_radix_tree(n, d_unique, out->codes, out->tree.prefix_n, out->tree.has_leaf_left,
                          out->tree.has_leaf_right, out->tree.left_child, out->tree.parent, s);
  if (e == cudaSuccess)
    e = launch_edge_scan(kEdgeAndScan, n, d_unique, out->tree.prefix_n, out->tree.parent,
                         out->edge_count, out->prefix_sum, d_max_slot, &L.scan, w + L.scan_off,
                         status, s);
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
    e = launch_octree(kOctMake | kOctLink | kOctFresh, a, oct_tags_carve(w + L.tags_off, a.cap),
                      status, s);
  }
  if (e == cudaSuccess) e = launch_publish_counts(d_unique, d_max_slot, status, out->d_counts, s);
  if (e == cudaSuccess && d_stats)
    e = cudaMemcpyAsync(d_stats, w + L.lsort_off + L.lp.stats_off, sizeof(LsortStats),
                        cudaMemcpyDeviceToDevice, s);
  return e == cudaSuccess ? OCT_OK : fail_cuda(e, "oct_build_octree_learned");
}

}  // extern "C"
