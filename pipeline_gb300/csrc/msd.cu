// Stages 2-3 of the whole build in MSD form, for large clouds whose keys
// spread evenly over the top digit (k_SimpleRadixSort + k_CountUnique,
// reference kernels/02_sort.cpp:13-58 and kernels/03_unique.cpp:2-16: the
// sorted unique codes are the same whichever way they are found).
//
//   gate     from the Morton kernel's top-digit histogram (bits 20..29): the
//            MSD form runs when n >= 2^22 and no top-digit bucket holds more
//            than 4x the mean; otherwise the LSD passes and the run-head
//            unique run. Both forms are launched; the unused one's kernels
//            return at once (a device flag each).
//   scatter  one unstable radix pass on the top digit: the LSD form's pass-0
//            launches, which take the top digit's shift, bases and split sums
//            when the MSD flag is set, so bucket b holds the keys
//            [b << 20, (b + 1) << 20) in any order;
//   buckets  one CTA per SM walks the buckets: a 2^20-bit bitmap (128 KiB of
//            shared memory) marks the bucket's keys; its set bits, read in
//            order, are the bucket's sorted unique keys (duplicates mark the
//            same bit), staged behind the bitmap and written over the front
//            of the bucket's own range;
//   pack     a scan of the unique counts, then one CTA per bucket copies its
//            run to its output offset with the delta of each code to the
//            next (the radix tree's input) and lowers the minima of the tree
//            tiles it touches: the same outputs as the LSD form's unique
//            stage.
#include <algorithm>

#include "kernels.cuh"
#include "tree.cuh"

namespace octgb {

constexpr int kMsdSpanBits = 20;                       // key bits below the top digit
constexpr int kMsdBuckets = 1 << (30 - kMsdSpanBits);  // 1,024
constexpr int kMsdWords = 1 << (kMsdSpanBits - 5);     // bitmap words per bucket
constexpr int kMsdThreads = 1024;
constexpr int kMsdStage = 24576;  // run keys staged in shared memory behind the bitmap
constexpr int kMsdWarpWords = kMsdWords / (kMsdThreads / 32);
constexpr int kMsdMinN = 1 << 22;
constexpr uint32_t kMsdSkew = 4;
constexpr int kPackThreads = 512;

static_assert(kMsdBuckets == kMsdThreads, "one gate thread per bucket");
static_assert(kMsdWarpWords == 32 * 32, "a warp's words are 32 rows of 32");

int msd_min_n() { return kMsdMinN; }
size_t msd_scratch_bytes() { return sizeof(uint32_t) * (3 * (size_t)kMsdBuckets + 1); }

__global__ void __launch_bounds__(kMsdBuckets)
    msd_gate_kernel(const uint32_t* __restrict__ top_hist, int n, uint32_t* __restrict__ flags) {
  chain_enter();
  __shared__ uint32_t s_max[kMsdBuckets / 32];
  const uint32_t m = __reduce_max_sync(0xffffffffu, top_hist[threadIdx.x]);
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t mx = 0;
    for (int w = 0; w < kMsdBuckets / 32; ++w) mx = max(mx, s_max[w]);
    const uint32_t mean = ((uint32_t)n + kMsdBuckets - 1) / kMsdBuckets;
    const bool msd = n >= kMsdMinN && mx <= kMsdSkew * mean;
    flags[0] = msd ? 1u : 0u;  // MSD form
    flags[1] = msd ? 0u : 1u;  // LSD form
  }
}

// Bitmap word x lives at x ^ (((x >> 5) & 7) << 2): the 32 words of a lane's
// 1,024-value chunk stay together, and the eight lanes of a 16-byte shared
// load phase read eight different bank groups.
__device__ __forceinline__ uint32_t msd_swz(uint32_t x) { return x ^ (((x >> 5) & 7u) << 2); }

__device__ __forceinline__ void msd_bucket(uint32_t* __restrict__ keys, uint32_t lo, uint32_t cnt,
                                           int b, uint32_t* bm, uint32_t* s_wsum,
                                           uint32_t* __restrict__ ucount,
                                           uint32_t* __restrict__ status, int tid, int lane,
                                           int w) {
  uint4* s_bm4 = reinterpret_cast<uint4*>(bm);
  for (int i = tid; i < kMsdWords / 4; i += kMsdThreads) s_bm4[i] = make_uint4(0u, 0u, 0u, 0u);
  __syncthreads();
  bool bad = false;
  constexpr int kBatch = 8;  // keys in flight per thread
  for (uint32_t i0 = 0; i0 < cnt; i0 += kBatch * kMsdThreads) {
    uint32_t k[kBatch];
#pragma unroll
    for (int q = 0; q < kBatch; ++q) {
      const uint32_t i = i0 + (uint32_t)(q * kMsdThreads + tid);
      k[q] = i < cnt ? keys[lo + i] : ((uint32_t)b << kMsdSpanBits);
    }
#pragma unroll
    for (int q = 0; q < kBatch; ++q) {
      const uint32_t i = i0 + (uint32_t)(q * kMsdThreads + tid);
      if (i >= cnt) continue;
      if ((k[q] >> kMsdSpanBits) != (uint32_t)b) {  // not this bucket's: never past the bitmap
        bad = true;
        continue;
      }
      const uint32_t v = k[q] & ((1u << kMsdSpanBits) - 1u);
      atomicOr(&bm[msd_swz(v >> 5)], 1u << (v & 31u));
    }
  }
  if (__syncthreads_or(bad) && tid == 0) raise_status(status, kStatusRange);
  // Thread tid owns chunk tid: values [tid * 1024, tid * 1024 + 1024), its 32
  // words read into registers in value order.
  const int c = tid;
  uint32_t wd[32];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint4 v = s_bm4[c * 8 + (j ^ (c & 7))];
    wd[4 * j] = v.x;
    wd[4 * j + 1] = v.y;
    wd[4 * j + 2] = v.z;
    wd[4 * j + 3] = v.w;
  }
  uint32_t own = 0, nz = 0;  // set bits, and the words that have any
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    own += __popc(wd[k]);
    nz |= (wd[k] != 0u ? 1u : 0u) << k;
  }
  uint32_t inc = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) s_wsum[w] = inc;
  if (tid == 0) bulk_wait_read();  // the previous bucket's copy has read the stage
  __syncthreads();
  uint32_t pos = inc - own, total = 0;
#pragma unroll 8
  for (int k = 0; k < kMsdThreads / 32; ++k) {
    const uint32_t v = s_wsum[k];
    if (k < w) pos += v;
    total += v;
  }
  if (tid == 0) ucount[b] = total;
  // Every key was read before the first barrier: the run overwrites the front
  // of the bucket's own range, staged behind the bitmap when it fits there
  // (kMsdStage keys), else written straight out. `total` is the same in
  // every thread, so the branch is uniform. A lane walks its own set bits in
  // one loop (words re-read from the bitmap), so a warp runs as many rounds
  // as its fullest lane has keys. The stage starts at the run's offset
  // within its 16-byte word, so the run's 16-byte words are the stage's.
  uint32_t* out = keys + lo;
  const uint32_t sh = lo & 3u;
  uint32_t* stage = bm + kMsdWords;
  const bool staged = total <= (uint32_t)kMsdStage;
  uint32_t* dst = staged ? stage + sh : out;
  const uint32_t kc = ((uint32_t)b << kMsdSpanBits) | ((uint32_t)c << 10);
  uint32_t bits = 0, kw = 0;
  for (uint32_t e = 0; e < own; ++e) {
    if (bits == 0u) {
      const int k = __ffs(nz) - 1;
      nz &= nz - 1u;
      kw = kc | ((uint32_t)k << 5);
      bits = bm[msd_swz((uint32_t)(c * 32 + k))];
    }
    const int bit = __ffs(bits) - 1;
    bits &= bits - 1u;
    dst[pos + e] = kw | (uint32_t)bit;
  }
  if (staged) {
    bulk_fence_writes();
    __syncthreads();
    // the aligned middle as one bulk copy (the TMA engine writes it while the
    // CTA goes on to the next bucket's bitmap), the ragged ends by threads
    const uint32_t h0 = min((4u - sh) & 3u, total);
    const uint32_t mid = (total - h0) & ~3u;
    if (tid == 0 && mid > 0) bulk_store_s2g(out + h0, stage + sh + h0, mid * 4u);
    if (tid < h0) out[tid] = stage[sh + tid];
    for (uint32_t i = h0 + mid + tid; i < total; i += kMsdThreads) out[i] = stage[sh + i];
  }
}

__global__ void __launch_bounds__(kMsdThreads, 1)
    msd_bucket_kernel(uint32_t* __restrict__ keys, const uint32_t* __restrict__ top_base,
                      const uint32_t* __restrict__ top_hist, uint32_t* __restrict__ ucount,
                      const uint32_t* __restrict__ gate, uint32_t* __restrict__ status) {
  chain_enter();
  if (*gate == 0) return;
  extern __shared__ uint4 s_bm4[];
  uint32_t* bm = reinterpret_cast<uint32_t*>(s_bm4);
  __shared__ uint32_t s_wsum[kMsdThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  // one CTA per SM (its shared memory) walks the buckets
  for (int b = blockIdx.x; b < kMsdBuckets; b += gridDim.x) {
    msd_bucket(keys, top_base[b], top_hist[b], b, bm, s_wsum, ucount, status, tid, lane, w);
    __syncthreads();  // the next bucket clears the bitmap
  }
  if (tid == 0) bulk_wait_all();  // the runs are written before the kernel ends
}

__global__ void __launch_bounds__(kMsdBuckets)
    msd_pack_scan_kernel(const uint32_t* __restrict__ ucount, uint32_t* __restrict__ uoff,
                         int* __restrict__ next_start, const uint32_t* __restrict__ top_base,
                         int* __restrict__ d_unique, TreeScratch S,
                         const uint32_t* __restrict__ gate) {
  chain_enter();
  if (*gate == 0) return;
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t total;
  __shared__ int s_ne[kMsdBuckets + 1];
  const int b = threadIdx.x;
  const uint32_t c = ucount[b];
  const uint32_t ex = block_exclusive_sum<kMsdBuckets>(c, warp_tot, &total);
  uoff[b] = ex;
  // the next bucket with keys after b (suffix minimum of the non-empty ids)
  s_ne[b] = c > 0 ? b : kMsdBuckets;
  if (b == 0) s_ne[kMsdBuckets] = kMsdBuckets;
  __syncthreads();
  for (int d = 1; d < kMsdBuckets; d <<= 1) {
    const int v = min(s_ne[b], s_ne[min(b + d, kMsdBuckets)]);
    __syncthreads();
    s_ne[b] = v;
    __syncthreads();
  }
  const int nb = s_ne[b + 1];
  next_start[b] = nb < kMsdBuckets ? (int)top_base[nb] : -1;
  if (b == 0) {
    uoff[kMsdBuckets] = total;
    *d_unique = (int)total;
  }
  // the tree scratch of the LSD form's unique stage: no tile sums yet, every
  // tile minimum absent until the pack lowers it
  const int pad = (int)align_up((size_t)S.tiles, kTtMinBlock);
  for (int k = b; k < pad; k += kMsdBuckets) S.tile_min[k] = (uint8_t)kTtAbsent;
  for (int k = b; k < S.tiles; k += kMsdBuckets) S.tile_sum[k] = 0;
}

constexpr int kPackTiles = 1028;  // tree tiles one bucket's run can touch (4x the mean of 2^20)

__device__ __forceinline__ void msd_pack_run(const uint32_t* __restrict__ keys, uint32_t start,
                                             uint32_t u, uint32_t o0, uint32_t U, int ns,
                                             uint32_t* __restrict__ codes, const TreeScratch& S,
                                             uint32_t* s_tmin, int tid) {
  const uint32_t* src = keys + start;
  const uint32_t after = ns >= 0 ? keys[ns] : 0u;  // read only when a code follows the run
  const uint32_t t0 = o0 / kTtTile;
  const uint32_t nt = min((o0 + u - 1) / kTtTile - t0 + 1, (uint32_t)kPackTiles);
  for (uint32_t k = tid; k < nt; k += kPackThreads) s_tmin[k] = kTtAbsent;
  __syncthreads();
  const uint32_t lane = tid & 31, warp = tid >> 5;
  constexpr uint32_t kRows = 8;  // a warp takes 8 x 32 consecutive codes per round
  constexpr uint32_t kSpan = kRows * 32;
  // whole warps iterate together (the shuffles and warp minima need every lane)
  for (uint32_t j0 = warp * kSpan; j0 < u; j0 += (kPackThreads / 32) * kSpan) {
    uint32_t k[kRows];
#pragma unroll
    for (uint32_t q = 0; q < kRows; ++q) {
      const uint32_t j = j0 + q * 32 + lane;
      k[q] = j < u ? src[j] : 0u;
    }
    // the code after this round's last: the next round's first, or the next run's
    const uint32_t jn = j0 + kSpan;
    const uint32_t tail = jn < u ? src[jn] : after;
    uint32_t ma = kTtAbsent, mb = kTtAbsent;
    const uint32_t ta = (o0 + j0) / kTtTile;  // the round's 256 positions: one tile or two
#pragma unroll
    for (uint32_t q = 0; q < kRows; ++q) {
      const uint32_t j = j0 + q * 32 + lane;
      const uint32_t o = o0 + j;
      const uint32_t down = __shfl_down_sync(0xffffffffu, k[q], 1);
      const uint32_t next_row = q + 1 < kRows ? __shfl_sync(0xffffffffu, k[q + 1 < kRows ? q + 1 : q], 0)
                                              : tail;
      const uint32_t nxt = j + 1u < u ? (lane < 31 ? down : next_row) : after;
      if (j < u) {
        codes[o] = k[q];
        if (o + 1u < U) {
          const uint32_t d = tt_delta(k[q], nxt);
          S.D[o] = (uint8_t)d;
          if (o / kTtTile == ta) ma = min(ma, d);
          else mb = min(mb, d);
        }
      }
    }
    ma = __reduce_min_sync(0xffffffffu, ma);
    mb = __reduce_min_sync(0xffffffffu, mb);
    if (lane == 0) {
      if (ma < kTtAbsent) {
        if (ta - t0 < nt) atomicMin(&s_tmin[ta - t0], ma);
        else atomic_min_u8(S.tile_min + ta, ma);  // beyond the shared table
      }
      if (mb < kTtAbsent) {
        if (ta + 1 - t0 < nt) atomicMin(&s_tmin[ta + 1 - t0], mb);
        else atomic_min_u8(S.tile_min + ta + 1, mb);
      }
    }
  }
  __syncthreads();
  for (uint32_t k = tid; k < nt; k += kPackThreads)
    if (s_tmin[k] < kTtAbsent) atomic_min_u8(S.tile_min + t0 + k, s_tmin[k]);
}

// A CTA per bucket (the loop serves any grid): a run goes to the codes from
// its output offset, with each code's delta to the next one (the next
// bucket's first code after the run's last) and the touched tree tiles'
// minima.
__global__ void __launch_bounds__(kPackThreads)
    msd_pack_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ top_base,
                    const uint32_t* __restrict__ ucount, const uint32_t* __restrict__ uoff,
                    const int* __restrict__ next_start, uint32_t* __restrict__ codes,
                    TreeScratch S, const uint32_t* __restrict__ gate) {
  chain_enter();
  if (*gate == 0) return;
  __shared__ uint32_t s_tmin[kPackTiles];
  const int tid = threadIdx.x;
  for (int b = blockIdx.x; b < kMsdBuckets; b += gridDim.x) {
    const uint32_t u = ucount[b];
    if (u != 0) msd_pack_run(keys, top_base[b], u, uoff[b], uoff[kMsdBuckets], next_start[b],
                             codes, S, s_tmin, tid);
    __syncthreads();  // s_tmin is the next run's
  }
}

cudaError_t launch_msd_gate(const uint32_t* top_hist, int n, uint32_t* flags, cudaStream_t s) {
  return launch_chained(msd_gate_kernel, dim3(1), dim3(kMsdBuckets), 0, s, top_hist, n, flags);
}

cudaError_t launch_msd_buckets(uint32_t* keys, const uint32_t* top_base, const uint32_t* top_hist,
                               void* scratch, const uint32_t* gate, uint32_t* status,
                               cudaStream_t s) {
  constexpr int smem = sizeof(uint32_t) * (kMsdWords + kMsdStage + 4);  // + the stage's shift
  const cudaError_t e = set_smem_limit(msd_bucket_kernel, smem);
  if (e != cudaSuccess) return e;
  uint32_t* ucount = static_cast<uint32_t*>(scratch);
  const int grid = std::min(kMsdBuckets, device_sm_count());  // one CTA fits an SM
  return launch_chained(msd_bucket_kernel, dim3(grid), dim3(kMsdThreads), smem, s, keys, top_base,
                        top_hist, ucount, gate, status);
}

cudaError_t launch_msd_pack(const uint32_t* keys, const uint32_t* top_base, int n,
                            uint32_t* codes_out, int* d_unique, void* scratch,
                            void* tree_scratch, const uint32_t* gate, cudaStream_t s) {
  uint32_t* ucount = static_cast<uint32_t*>(scratch);
  uint32_t* uoff = ucount + kMsdBuckets;
  int* next_start = reinterpret_cast<int*>(uoff + kMsdBuckets + 1);
  const TreeScratch S = tree_scratch_carve(tree_scratch, n);
  cudaError_t e = launch_chained(msd_pack_scan_kernel, dim3(1), dim3(kMsdBuckets), 0, s, ucount,
                                 uoff, next_start, top_base, d_unique, S, gate);
  if (e != cudaSuccess) return e;
  return launch_chained(msd_pack_kernel, dim3(kMsdBuckets), dim3(kPackThreads), 0, s, keys,
                        top_base, ucount, uoff, next_start, codes_out, S, gate);
}

}  // namespace octgb
