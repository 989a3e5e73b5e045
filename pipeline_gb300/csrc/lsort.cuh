// Learned bucketed sort + unique: plan and launch interface.
#pragma once

#include "learned.cuh"

namespace octgb {

// Device-side statistics of one learned sort (in the zeroed workspace).
struct LsortStats {
  uint32_t fallback;        // 1: the OneSweep path produced the result
  uint32_t failed_buckets;  // buckets that fit neither bucket form
  uint32_t overflow_keys;   // keys in buckets above the bitonic capacity
  uint32_t max_bucket;      // largest bucket
  uint32_t n;
  float overflow_frac;      // overflow_keys / n
  uint32_t skip;            // set after the bin pass: the bucket stage does not run
  uint32_t bitmap_buckets;  // buckets sorted through a shared-memory bitmap
  uint32_t radix_buckets;   // ... through the shared-memory radix sort
  uint32_t bitonic_buckets; // ... through the bitonic sort
  uint32_t pad[2];
};
static_assert(sizeof(LsortStats) == 48, "LsortStats is 12 words");

struct LsortPlan {
  int n, nb;
  LcdfLayout L;
  SortPlan fallback_sort;
  ScanPlan fallback_unique;
  size_t stats_off, sort_ctrl_off, uniq_ctrl_off, zero_bytes;
  size_t cursor_off, starts_off, counts_off, ucount_off, uoff_off, bkeys_off, alt_off, bytes;
  uint32_t cap;  // keys per bucket range of bkeys
};

LsortPlan lsort_plan(int n, int nb, int max_segments);
size_t lsort_hist_smem(int nb, int max_segments);
constexpr int kLsortMaxSmem = 227 * 1024;  // dynamic shared memory per CTA on sm_103

// Sorted unique keys into `out`, U into *d_unique. With pts != nullptr the
// keys are Morton-encoded from the points first (into `keys`).
cudaError_t launch_lsort(const float4* pts, uint32_t* keys, int n, float min_coord, float range,
                         const char* blob, const LsortPlan& p, char* ws, float threshold,
                         uint32_t* out, int* d_unique, uint32_t* status, cudaStream_t s,
                         Recorder* rec);

// Learned bucket sort of a batch of clouds: each cloud's range of `out`
// receives its sorted unique keys followed by copies of its largest key
// (sorted keys, for the batched unique stage), unless a bucket fits none of
// the bucket forms, which sets stats->fallback and leaves `out` to a sort
// gated on that flag. `keys` is not modified.
struct LbatchArgs {
  const uint32_t* keys;      // cloud-concatenated Morton codes
  uint32_t* out;             // cloud-concatenated sorted codes
  const int4* tiles;         // sort tiles {lo, hi, cloud, the cloud's first tile}
  int n_tiles;
  const int* start;          // [C + 1] cloud starts
  const int* cloud_tile0;    // [C + 1] first tile of each cloud
  int C;
  int n;                     // keys in the batch
  const char* blob;          // the model
  LcdfLayout L;
  int nb;                    // buckets per cloud
  void* scratch;             // lbatch_scratch_bytes(n_tiles, C, nb, n), not zeroed
  LsortStats* stats;         // zeroed before the call (fallback, max_bucket, bucket forms)
};
size_t lbatch_scratch_bytes(int n_tiles, int n_clouds, int nb, int n);
cudaError_t launch_lbatch_sort(const LbatchArgs& a, cudaStream_t s);

}  // namespace octgb
