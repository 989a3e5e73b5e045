// Internal launch interface shared by the kernel translation units and the
// C-ABI layer (api.cu). Nothing here is exported from the shared library.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "common.cuh"
#include "octree_gb300.h"

namespace octgb {

__host__ __device__ static inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Optional per-launch event recording (timed builds): mark() records the next
// caller event on the stream after a launch.
struct Recorder {
  cudaEvent_t* events = nullptr;
  int n = 0;
  int k = 0;
  cudaError_t err = cudaSuccess;
  void mark(cudaStream_t s) {
    if (k < n && err == cudaSuccess) err = cudaEventRecord(events[k], s);
    ++k;
  }
};
static inline void mark(Recorder* r, cudaStream_t s) {
  if (r) r->mark(s);
}

// SM count of the current device (cached per device).
int device_sm_count();

// Whether launch_chained may set the programmatic-serialization attribute:
// yes unless the environment sets OCT_PDL=0 (read once per process).
bool chained_launches();

// True while `s` is being captured into a CUDA graph (a failed query, e.g.
// on the legacy stream during another thread's global capture, counts as
// not capturing and its error is cleared).
static inline bool stream_capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return cs == cudaStreamCaptureStatusActive;
}

// Launch of a kernel whose body starts with chain_enter() (common.cuh). While
// the stream is captured into a CUDA graph the launch carries programmatic
// stream serialization, so in the graph's replays the kernel's CTAs may be
// scheduled during the tail of the kernel before it and wait there on the
// device, without a full launch gap between them; launched directly on a
// stream (timed builds, pipelines overlapping copies on other streams) it is
// a plain launch. Results are the same either way.
template <typename... P, typename... A>
static inline cudaError_t launch_chained(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem,
                                         cudaStream_t s, A&&... args) {
  cudaLaunchConfig_t c = {};
  c.gridDim = grid;
  c.blockDim = block;
  c.dynamicSmemBytes = smem;
  c.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  c.attrs = at;
  c.numAttrs = chained_launches() && stream_capturing(s) ? 1 : 0;
  return cudaLaunchKernelEx(&c, kernel, static_cast<P>(args)...);
}

// Raises func's dynamic shared-memory limit to at least `bytes` on the
// current device (once per device and kernel; kernel attributes are per
// device context).
cudaError_t set_smem_limit(const void* func, int bytes);
template <typename F>
static inline cudaError_t set_smem_limit(F* func, int bytes) {
  return set_smem_limit(reinterpret_cast<const void*>(func), bytes);
}

// Sets the text oct_last_error() returns on this thread.
void set_last_error(const char* msg);

// ---- diagnostics ---------------------------------------------------------
// One look-back wait on a tile whose predecessor never publishes (the sort's
// digit look-back over 2 x 1024 words, or the unique / prefix-sum warp
// look-back over 2 words), bounded by limit_ns.
cudaError_t launch_diag_sort_wait(uint32_t* lookback, uint32_t* status,
                                  unsigned long long limit_ns, cudaStream_t s);
cudaError_t launch_diag_scan_wait(unsigned long long* lb, uint32_t* status,
                                  unsigned long long limit_ns, cudaStream_t s);

// ---- sort ----------------------------------------------------------------
// Tunable shape of the radix sort (chosen by the autotuner or the default).
struct SortConfig {
  int radix_bits;  // 10 (3 passes over 30-bit keys) or 8
  int warps;       // warps per tile CTA (16)
  int items;       // keys per thread (16 or 24)
  int scan;        // 0: decoupled look-back (OneSweep); 1: tile histograms + tile scan
};

struct SortPlan {
  int n;
  int radix_bits;
  int passes;
  int bins;
  int tile;
  int tiles;
  SortConfig cfg;
  size_t hist_off, counter_off, lookback_off, tile_part_off, base_off, tile_hist_off;
  size_t zero_bytes;  // [0, zero_bytes) is cleared before each sort
  size_t bytes;       // whole control block
};

SortPlan sort_plan(int n, int key_bits);
SortPlan sort_plan_cfg(int n, int key_bits, SortConfig cfg);
// One digit pass (batched sorts: tile descriptors int4{first, end, cloud,
// first tile of cloud} and their count; nullptr / 0 for a single array).
// A pass launch that serves as either of two passes, chosen on the device:
// when *flag != 0 the pass kernel uses this shift and these digit bases, and
// an unstable reduce-then-scan pass takes its digit runs' places from the
// cursors in `part` (one per digit, kCursorStride words apart, zeroed before
// the sort) instead of the tile scan.
struct DigitAlt {
  const uint32_t* flag = nullptr;
  int shift = 0;
  const uint32_t* base = nullptr;
  uint32_t* part = nullptr;
};
constexpr int kCursorStride = 16;
cudaError_t launch_pass(const SortPlan& p, bool stable, const uint32_t* src, uint32_t* dst,
                        int shift, const uint32_t* base, uint32_t* lookback, uint32_t* counter,
                        const uint32_t* tile_prefix, uint32_t* status, const uint32_t* gate,
                        cudaStream_t s, const int4* tdesc, int tiles, DigitAlt alt = DigitAlt{});
cudaError_t launch_tile_hist(int radix_bits, const uint32_t* keys, int n, int shift,
                             const int4* tdesc, int tiles, uint32_t* th, cudaStream_t s,
                             const uint32_t* gate = nullptr);
void set_sort_config(const SortConfig& c);
SortConfig get_sort_config();

// Morton encode; with plan != nullptr also accumulates the plan's digit
// histograms into the zeroed control block ctrl.
cudaError_t launch_morton(const float4* pts, uint32_t* keys, long long n, float min_coord,
                          float range, const SortPlan* plan, void* ctrl, uint32_t* status,
                          cudaStream_t s);
cudaError_t launch_histogram(const uint32_t* keys, const SortPlan* plan, void* ctrl,
                             cudaStream_t s);
cudaError_t launch_sort_passes(uint32_t* keys, uint32_t* alt, const SortPlan* plan, void* ctrl,
                               uint32_t* status, cudaStream_t s, uint32_t** result,
                               Recorder* rec = nullptr);
// Gated forms: the kernels return at once unless *gate != 0 (device flag).
cudaError_t launch_histogram_gated(const uint32_t* keys, const SortPlan* plan, void* ctrl,
                                   const uint32_t* gate, cudaStream_t s);
cudaError_t launch_sort_passes_gated(uint32_t* keys, uint32_t* alt, const SortPlan* plan,
                                     void* ctrl, uint32_t* status, const uint32_t* gate,
                                     cudaStream_t s, uint32_t** result);
// The digit bases (exclusive scans of the Morton kernel's histograms), always
// run; then the LSD passes. With msd_flag (device): pass 0's launches do the
// MSD form's top-digit scatter instead when *msd_flag != 0, and passes 1..
// are gated on lsd_flag.
cudaError_t launch_sort_passes_split(uint32_t* keys, uint32_t* alt, const SortPlan* plan,
                                     void* ctrl, uint32_t* status, const uint32_t* msd_flag,
                                     const uint32_t* lsd_flag, cudaStream_t s, uint32_t** result,
                                     Recorder* rec);

// ---- MSD form of stages 2-3 (whole builds of large, even clouds) ----------
// The form is chosen on the device from the top-digit histogram: flags[0]
// set runs the MSD kernels, flags[1] set the LSD passes and unique.
int msd_min_n();
size_t msd_scratch_bytes();
bool msd_plan_ok(const SortPlan& p);  // 10-bit digits, 3 passes, reduce-then-scan
cudaError_t launch_msd_gate(const uint32_t* top_hist, int n, uint32_t* flags, cudaStream_t s);
// The sorted unique keys of every top-digit bucket over the front of its
// range; the counts go to the scratch.
cudaError_t launch_msd_buckets(uint32_t* keys, const uint32_t* top_base, const uint32_t* top_hist,
                               void* scratch, const uint32_t* gate, uint32_t* status,
                               cudaStream_t s);
// Packs the bucket runs: codes, U to *d_unique, the adjacent deltas and tile
// minima into the tree scratch (as launch_unique_deltas leaves them).
cudaError_t launch_msd_pack(const uint32_t* keys, const uint32_t* top_base, int n,
                            uint32_t* codes_out, int* d_unique, void* scratch,
                            void* tree_scratch, const uint32_t* gate, cudaStream_t s);

// ---- unique --------------------------------------------------------------
struct ScanPlan {
  int n;
  int tile;
  int tiles;
  size_t counter_off, lookback_off;
  size_t bytes;  // control block, zeroed before each launch
};
ScanPlan unique_plan(int n);
// Compacts runs of equal keys of src[0, n) into dst (dst == src allowed);
// writes U to *d_count.
cudaError_t launch_unique(const uint32_t* src, uint32_t* dst, int n, int* d_count,
                          const ScanPlan* plan, void* ctrl, uint32_t* status, cudaStream_t s);
cudaError_t launch_unique_gated(const uint32_t* src, uint32_t* dst, int n, int* d_count,
                                const ScanPlan* plan, void* ctrl, uint32_t* status,
                                const uint32_t* gate, cudaStream_t s);

// ---- radix tree, edge count, prefix sum -----------------------------------
// n_nodes from the host (n_host) or, when d_unique != nullptr, as *d_unique - 1.
cudaError_t launch_radix_tree(int n_host, const int* d_unique, const uint32_t* codes,
                              uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr, int* left_child,
                              int* parent, cudaStream_t s);

// The same outputs for strictly increasing codes below 2^31 (the build's own
// sorted unique Morton codes), from the adjacent deltas; with ec != nullptr
// also the edge counts. scratch: tree_scratch_bytes(n_host), 256-aligned.
struct TreeScratch {
  uint8_t* D;          // [tiles * 4096] adjacent deltas, tile-major
  uint8_t* tile_min;   // [tiles rounded up to 512] smallest D of the tile
  int* tile_sum;       // [tiles] sum of the edge counts of the tile's 4,096 nodes
  uint32_t* tile_prefix;  // [tiles] exclusive prefix of tile_sum
  int* tile_heads;     // [tiles] run heads of a 4,096-key tile of the sorted keys
  uint32_t* tile_upos; // [tiles] exclusive prefix of tile_heads
  int tiles;
};
size_t tree_scratch_bytes(int n_host);
TreeScratch tree_scratch_carve(void* base, int n_host);
// Stage 3 fused with the deltas for the whole-cloud build: the run heads of the
// sorted keys are counted per 4,096-key tile and scanned (no look-back); the
// compaction writes the unique codes, U to *d_unique and, for each unique code
// but the first, the delta to the one before it into the tree scratch (and the
// tiles' smallest deltas), so only tree_nodes_kernel remains of stage 4.
cudaError_t launch_unique_deltas(const uint32_t* sorted, int n, uint32_t* codes_out, int* d_unique,
                                 void* tree_scratch, cudaStream_t s,
                                 const uint32_t* gate = nullptr);
// The same for batched clouds over their 4,096-key tiles (descriptors
// {first, end, cloud, first tile of cloud}): each cloud's codes from its
// start, its U to unique_c[cloud], its deltas in its own tree tiles.
cudaError_t launch_batch_unique_deltas(const uint32_t* sorted, const int4* tiles, int n_tiles,
                                       const int* start, uint32_t* codes_out, int* unique_c,
                                       void* scratch, cudaStream_t s);
cudaError_t launch_batch_radix_tree_from_deltas(const int4* tiles, int n_tiles, const int* start,
                                                const int* unique_c, const uint32_t* codes,
                                                uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                                                int* left_child, int* parent, int* ec,
                                                void* scratch, cudaStream_t s);
// The radix tree (and edge counts) from deltas already in the scratch.
cudaError_t launch_radix_tree_from_deltas(int n_host, const int* d_unique, const uint32_t* codes,
                                          uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                                          int* left_child, int* parent, int* ec, void* scratch,
                                          cudaStream_t s);
// Exclusive scan of `tiles` counts into prefix (one CTA); total to *total_out.
cudaError_t launch_tile_counts_scan(int tiles, const int* counts, uint32_t* prefix,
                                    int* total_out, cudaStream_t s,
                                    const uint32_t* gate = nullptr);
size_t tree_scratch_bytes_tiles(int tiles);
TreeScratch tree_scratch_carve_tiles(void* base, int tiles);
// Batched clouds: tiles {first, end, cloud, first tile of cloud} of 4,096
// positions that never cross clouds; start[C+1]; U per cloud on the device.
cudaError_t launch_batch_radix_tree(const int4* tiles, int n_tiles, const int* start,
                                    const int* unique_c, const uint32_t* codes, uint8_t* prefix_n,
                                    uint8_t* hll, uint8_t* hlr, int* left_child, int* parent,
                                    int* ec, void* scratch, cudaStream_t s);
cudaError_t launch_radix_tree_sorted(int n_host, const int* d_unique, const uint32_t* codes,
                                     uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                                     int* left_child, int* parent, int* ec, void* scratch,
                                     cudaStream_t s);

ScanPlan edge_scan_plan(int n);
enum EdgeScanMode { kEdgeOnly = 1, kScanOnly = 2, kEdgeAndScan = 3 };
// kEdgeOnly: ec = edge counts. kScanOnly: ps = inclusive scan of ec.
// kEdgeAndScan: both, fused. With d_max_slot != nullptr, atomically raises
// *d_max_slot to the largest octree slot stages 7-8 will write.
cudaError_t launch_edge_scan(int mode, int n_host, const int* d_unique, const uint8_t* prefix_n,
                             const int* parent, int* ec, int* ps, int* d_max_slot,
                             const ScanPlan* plan, void* ctrl, uint32_t* status, cudaStream_t s);

// ---- octree --------------------------------------------------------------
struct OctTags {
  uint32_t* child;  // [cap * 8] winning write tag per (slot, child)
  uint32_t* owner;  // [cap] last radix node that wrote corner / cell_size
  uint32_t* mask;   // [cap] OR of SetChild bits
  int cap;
};
size_t oct_tags_bytes(int cap);
OctTags oct_tags_carve(void* base, int cap);

// Zeroes the tags of slots [lo, hi] (inclusive) with `nthreads` threads of
// index `tid`: consecutive threads take consecutive 16-byte child words, so
// every warp store fills whole sectors.
__device__ __forceinline__ void clear_tag_range(const OctTags& t, size_t lo, size_t hi, int tid,
                                                int nthreads) {
  if (hi < lo) return;
  uint4* c4 = reinterpret_cast<uint4*>(t.child);
  for (size_t q = 2 * lo + (size_t)tid; q < 2 * hi + 2; q += (size_t)nthreads)
    c4[q] = make_uint4(0, 0, 0, 0);
  for (size_t p = lo + (size_t)tid; p <= hi; p += (size_t)nthreads) {
    t.owner[p] = 0;
    t.mask[p] = 0;
  }
}

enum OctMode { kOctMake = 1, kOctLink = 2, kOctFresh = 4 };

struct OctArgs {
  oct_node* nodes;
  int cap;
  const int* offsets;      // prefix sum
  const int* counts;       // edge count
  const uint32_t* codes;   // sorted unique codes
  const uint8_t* prefix_n;
  const uint8_t* hll;
  const uint8_t* hlr;
  const int* parent;
  const int* left_child;
  float min_coord, range;
  int n_brt_host;          // used when d_unique == nullptr
  const int* d_unique;     // U on the device (n_brt = U - 1)
  int n_oct_host;          // used when d_max_slot == nullptr
  const int* d_max_slot;   // largest slot on the device (n_oct = max_slot + 1)
};
// tags_clear: the tags of [0, M) are already zero (launch_prefix_sum_clear_tags).
cudaError_t launch_octree(int mode, const OctArgs& a, const OctTags& t, uint32_t* status,
                          cudaStream_t s, Recorder* rec = nullptr, bool tags_clear = false);

// Inclusive prefix sum of the edge counts written by launch_radix_tree_sorted
// (which also summed them per 4,096-node tile into the scratch) that also
// clears the octree tags of every slot stages 7-8 can touch, up to the tags'
// capacity: one small kernel scans the tile sums, then every tile scans its
// own nodes from its prefix (no inter-tile waits).
// Exclusive scan of tiles per-tile sums (one CTA).
cudaError_t launch_tile_sums_scan(int tiles, const int* tile_sum, uint32_t* tile_prefix,
                                  cudaStream_t s);

cudaError_t launch_prefix_sum_clear_tags(int n_host, const int* d_unique, int* ec, int* ps,
                                         int* d_max_slot, void* tree_scratch, uint32_t* status,
                                         const OctTags& tags, cudaStream_t s);

// Copies U, B, M, status into out[4] (device).
cudaError_t launch_publish_counts(const int* d_unique, const int* d_max_slot,
                                  const uint32_t* status, int* out, cudaStream_t s);

}  // namespace octgb
