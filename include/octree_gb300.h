/*
 * octree_gb300.h — C ABI of the GB300 (sm_103a) octree-build library
 * (libpipeline_gb300.so).
 *
 * Drop-in for the seven-stage octree build of ucsc-redwood/pipeline: Morton
 * encode, radix sort, unique, Karras radix tree, edge count, prefix sum and
 * octree nodes (+ leaf links). Each stage entry point below names the
 * reference function it replaces (paths within the reference project).
 *
 * Conventions
 *  - Plain C: pointers, sizes, a CUDA stream (may be NULL = legacy stream).
 *  - Pointers are DEVICE pointers (cudaMalloc / cudaMallocManaged) unless a
 *    function says otherwise. The caller owns every buffer, as in the
 *    reference (include/shared/types.h:5-8).
 *  - Entry points are asynchronous on the given stream and return an
 *    oct_status for argument / launch errors. Conditions found on the device
 *    (a look-back wait that ran out its bound, a coordinate outside
 *    [min, min + range], a too-small octree capacity) are OR-ed into an
 *    optional device status word (OCT_STATUS_* bits); no call aborts or traps.
 *  - Scratch comes from a caller workspace whose size the matching
 *    *_workspace_bytes() function returns (256-byte aligned base required).
 *  - Results are bit-identical to the reference's CPU implementation on the
 *    same inputs, run with one thread, under these conventions where the
 *    reference leaves behaviour undefined:
 *      O1  the radix tree has n_nodes = U - 1 nodes (apps/cpu_demo/main.cpp:95);
 *      O3  the octree has M = 1 + the largest slot stages 7-8 write
 *          (= prefix_sum[U-2] + 1 whenever the reference stays in bounds);
 *      O4  outputs start zeroed (OctNodes, parent[]);
 *      O6  stages 7-8 take the values a sequential ascending-node run leaves;
 *      O7  a leaf-link walk stops at radix node 0 (the reference never returns);
 *      O10 a shift by a negative count (leaf level 11) shifts by count mod 32;
 *      O11 a one-node tree (U = 2) uses clz(0) = 32 and drops the
 *          out-of-range parent write.
 */
#ifndef OCTREE_GB300_H
#define OCTREE_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define OCT_API __attribute__((visibility("default")))
#else
#define OCT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without including the CUDA headers. */
typedef struct CUstream_st* oct_stream_t;

/* glm::vec4 as the reference stores points and corners: four floats, 16 B. */
typedef struct oct_vec4 {
  float x, y, z, w;
} oct_vec4;

/* OctNode (reference include/shared/types.h:28-34), 60 bytes. */
typedef struct oct_node {
  int32_t children[8];
  oct_vec4 corner;
  float cell_size;
  int32_t child_node_mask;
  int32_t child_leaf_mask;
} oct_node;

/* RadixTreeData (reference include/shared/types.h:14-21); bool is 1 byte. */
typedef struct oct_radix_tree {
  int32_t n_nodes;
  uint8_t* prefix_n;
  uint8_t* has_leaf_left;
  uint8_t* has_leaf_right;
  int32_t* left_child;
  int32_t* parent;
} oct_radix_tree;

typedef enum oct_status {
  OCT_OK = 0,
  OCT_ERR_INVALID_ARG = 1, /* bad size, null pointer, misaligned buffer */
  OCT_ERR_WORKSPACE = 2,   /* workspace smaller than *_workspace_bytes() */
  OCT_ERR_CUDA = 3,        /* a CUDA runtime call or launch failed */
  OCT_ERR_DEVICE = 4,      /* the device status word is non-zero (sync calls) */
  OCT_ERR_CAPACITY = 5,    /* octree node buffer too small (sync calls) */
  OCT_ERR_TOO_LARGE = 6    /* size above a fixed limit (oct_sort_keys_noalloc,
                              OCT_MAX_OCTREE_NODES) */
} oct_status;

/* Device status word bits. */
#define OCT_STATUS_SPIN_TIMEOUT 1u /* a decoupled look-back wait gave up */
#define OCT_STATUS_WALK_LIMIT 2u   /* a radix-tree parent walk exceeded 64 steps */
#define OCT_STATUS_RANGE 4u        /* a coordinate outside [min, min + range] or NaN */
#define OCT_STATUS_CAPACITY 8u     /* octree needs more nodes than the buffer holds */

/* Largest point / key count accepted (counts travel in 30-bit fields). */
#define OCT_MAX_N ((1 << 30) - 1)

/* Largest radix-node count the octree stages (7-8) accept: their write tags
 * carry the radix node's index in 27 bits. Whole builds with an octree take
 * up to OCT_MAX_OCTREE_NODES + 1 points per cloud. */
#define OCT_MAX_OCTREE_NODES ((1 << 27) - 1)

/* Library version and the device architecture it was built for (e.g. 1033 = sm_103a). */
OCT_API int oct_version(void);
OCT_API int oct_built_arch(void);
/* Last CUDA error string seen by the library on this thread ("" if none). */
OCT_API const char* oct_last_error(void);

/* ----------------------------------------------------------------------- */
/* Stage 0 (host): input generator. Replaces k_InitRandomVec4               */
/* (include/kernels/00_init.hpp:10-11): n points drawn from std::mt19937     */
/* (seed) through std::uniform_real_distribution<float>(min, min + range),   */
/* z drawn first, then y, then x (GCC's argument order); w = 1. `out` is a   */
/* HOST pointer.                                                             */
/* ----------------------------------------------------------------------- */
OCT_API void oct_init_random_vec4(oct_vec4* out, int n, float min_coord, float range, int seed);

/* Stage 0 (device): key sequences. Replace k_InitDescending and            */
/* k_InitAscending (include/kernels/00_init.hpp:5-7, kernels/00_init.cpp:5-17)*/
/* : keys[i] = n - i, or keys[i] = i, for i in [0, n). d_keys: DEVICE       */
/* pointer. Asynchronous on `stream`.                                        */
OCT_API int oct_init_descending(uint32_t* d_keys, int n, oct_stream_t stream);
OCT_API int oct_init_ascending(uint32_t* d_keys, int n, oct_stream_t stream);

/* Stage 0 (device): the reference's device generator gpu::k_InitRandomVec4  */
/* (include/cuda/kernels/00_init.cuh:7-8, kernels/cuda/00_init.cu:11-50) as  */
/* its driver launches it (apps/gpu_demo/main.cu:168-175, one element per    */
/* thread): element i seeds four states from (4i + k) * seed, takes one step */
/* of the hybrid Tausworthe/LCG generator and maps 24 bits of z1^z2, z2^z3,  */
/* z3^z4, z1^z4 to fma(u / 2^24, range, min) (x, y, z, w; w is random too).  */
/* d_points: DEVICE pointer, 16-byte aligned. Asynchronous on `stream`.      */
OCT_API int oct_init_random_vec4_device(oct_vec4* d_points, int n, float min_coord, float range,
                                        int seed, oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Stage 1: Morton encode. Replaces k_ComputeMortonCode                     */
/* (include/kernels/01_morton.hpp:9-13; GPU kernels/cuda/01_morton.cu:8-19).*/
/* keys[i] = 30-bit Morton code of points[i] (w ignored).                   */
/* ----------------------------------------------------------------------- */
OCT_API int oct_morton_encode(const oct_vec4* points, uint32_t* keys, int64_t n, float min_coord,
                      float range, uint32_t* d_status, oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Stage 2: sort keys ascending, in place. Replaces k_SimpleRadixSort       */
/* (include/kernels/02_sort.hpp:6-7) and the GPU OneSweep dispatch          */
/* (apps/gpu_demo/main.cu:63-125). key_bits: significant low bits of every  */
/* key (30 for Morton codes, 32 for arbitrary keys). keys_alt: n-entry      */
/* scratch (the reference's keys_alt / OneSweepData::u_sort_alt).           */
/* ----------------------------------------------------------------------- */
OCT_API size_t oct_sort_workspace_bytes(int n, int key_bits);
OCT_API int oct_sort_keys(uint32_t* keys, uint32_t* keys_alt, int n, int key_bits, void* workspace,
                  size_t workspace_bytes, uint32_t* d_status, oct_stream_t stream);

/* Allocation-free variant of oct_sort_keys, for callers that cannot call
 * cudaMalloc (device memory owned by another allocator or a fixed pool; frame
 * loops where an allocation would stall the device). No counterpart in the
 * reference. Same keys / keys_alt / key_bits semantics; the scratch lives in
 * a fixed 6.5 MiB __device__ array inside the library, which every GPU that
 * loads the library holds until exit. n above OCT_NOALLOC_SORT_MAX_KEYS
 * returns OCT_ERR_TOO_LARGE. The first call on a device sets up the array's
 * address; make it before any stream capture. The address is kept for the
 * life of the process, so cudaDeviceReset on that device after the first
 * call is not supported. Several devices in one process are supported (each
 * gets its own array). Calls share the array: calls that overlap on the GPU
 * race. */
#define OCT_NOALLOC_SORT_MAX_KEYS (1 << 22)
#define OCT_NOALLOC_SORT_SCRATCH_BYTES (6815744u)
OCT_API int oct_sort_keys_noalloc(uint32_t* keys, uint32_t* keys_alt, int n, int key_bits,
                                  uint32_t* d_status, oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Stage 3: unique. Replaces k_CountUnique (include/kernels/03_unique.hpp:4,*/
/* kernels/03_unique.cpp:2-16): compacts runs of equal keys in place and    */
/* writes U to *d_n_unique (device int). keys[U, n) keep their old values.  */
/* ----------------------------------------------------------------------- */
OCT_API size_t oct_unique_workspace_bytes(int n);
OCT_API int oct_unique(uint32_t* keys, int n, int32_t* d_n_unique, void* workspace, size_t workspace_bytes,
               uint32_t* d_status, oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Stage 4: Karras radix tree over codes[0..n_nodes]. Replaces              */
/* k_BuildRadixTree (include/kernels/04_radix_tree.hpp:5-11). n_nodes is    */
/* U - 1. parent[] entries no node writes (parent[0], and parent[n-1] when  */
/* the root spans one key short) are set to 0.                              */
/* ----------------------------------------------------------------------- */
OCT_API int oct_build_radix_tree(int n_nodes, const uint32_t* codes, uint8_t* prefix_n,
                         uint8_t* has_leaf_left, uint8_t* has_leaf_right, int32_t* left_child,
                         int32_t* parent, oct_stream_t stream);

/* The same stage for strictly increasing codes below 2^31 (what stages 1-3 */
/* produce), built from the deltas of adjacent codes instead of per-node     */
/* searches; identical outputs for such codes (other inputs: unspecified     */
/* values, no out-of-bounds access). With edge_count != NULL it also writes  */
/* stage 5's edge counts (k_EdgeCount, include/kernels/05_edge_count.hpp:5-8)*/
/* for the same tree. workspace: oct_radix_tree_sorted_workspace_bytes(),    */
/* 256-byte aligned.                                                          */
/* ----------------------------------------------------------------------- */
OCT_API size_t oct_radix_tree_sorted_workspace_bytes(int n_nodes);
OCT_API int oct_build_radix_tree_sorted(int n_nodes, const uint32_t* codes, uint8_t* prefix_n,
                                uint8_t* has_leaf_left, uint8_t* has_leaf_right,
                                int32_t* left_child, int32_t* parent, int32_t* edge_count,
                                void* workspace, size_t workspace_bytes, oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Stage 5: edge count. Replaces k_EdgeCount                                 */
/* (include/kernels/05_edge_count.hpp:5-8): ec[0] = 0,                       */
/* ec[i] = prefix_n[i]/3 - prefix_n[parent[i]]/3.                            */
/* ----------------------------------------------------------------------- */
OCT_API int oct_edge_count(const uint8_t* prefix_n, const int32_t* parent, int32_t* edge_count,
                   int n_nodes, oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Stage 6: inclusive prefix sum. Replaces k_PartialSum                      */
/* (include/kernels/06_partial_sum.hpp:6-9) over data[0, n).                 */
/* ----------------------------------------------------------------------- */
OCT_API size_t oct_prefix_sum_workspace_bytes(int n);
OCT_API int oct_prefix_sum(const int32_t* data, int n, int32_t* out, void* workspace,
                   size_t workspace_bytes, uint32_t* d_status, oct_stream_t stream);

/* Number of octree nodes stages 7-8 need for this tree (O3): one past the
 * largest slot they write. Asynchronous: writes the count to the device int
 * *n_oct_nodes on the stream (the host reads it after the stream drains, as
 * apps/cpu_demo/main.cpp:120 reads num_oct_nodes). */
OCT_API int oct_octree_node_count(const int32_t* edge_count, const int32_t* prefix_sum,
                                  int n_nodes, int32_t* n_oct_nodes, oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Stage 7: octree nodes. Replaces k_MakeOctNodes                            */
/* (include/kernels/07_octree.hpp:5-14, shared/oct.h:24-90). Applies the     */
/* writes of radix nodes 1..n_nodes-1 to nodes[0, n_oct_nodes) in the order  */
/* a one-thread reference run makes them; the caller initialises nodes      */
/* (zeroed, root at slot 0) as apps/cpu_demo/main.cpp:123-132 does, or uses  */
/* oct_octree_root_init.                                                     */
/* ----------------------------------------------------------------------- */
OCT_API size_t oct_octree_workspace_bytes(int n_oct_nodes);
OCT_API int oct_octree_root_init(oct_node* nodes, const uint32_t* codes, const uint8_t* prefix_n,
                         float min_coord, float range, oct_stream_t stream);
OCT_API int oct_make_oct_nodes(oct_node* nodes, int n_oct_nodes, const int32_t* node_offsets,
                       const int32_t* rt_node_counts, const uint32_t* codes,
                       const uint8_t* rt_prefix_n, const int32_t* rt_parents, float min_coord,
                       float range, int n_nodes, void* workspace, size_t workspace_bytes,
                       uint32_t* d_status, oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Stage 8: leaf links. Replaces k_LinkLeafNodes                             */
/* (include/kernels/07_octree.hpp:16-25, shared/oct.h:92-134).               */
/* ----------------------------------------------------------------------- */
OCT_API int oct_link_leaf_nodes(oct_node* nodes, int n_oct_nodes, const int32_t* node_offsets,
                        const int32_t* rt_node_counts, const uint32_t* codes,
                        const uint8_t* rt_has_leaf_left, const uint8_t* rt_has_leaf_right,
                        const uint8_t* rt_prefix_n, const int32_t* rt_parents,
                        const int32_t* rt_left_child, int n_nodes, void* workspace,
                        size_t workspace_bytes, uint32_t* d_status, oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Whole build: stages 1-8 in the order of apps/cpu_demo/main.cpp:72-154,    */
/* all sizes kept on the device (no host round trip, CUDA-graph capturable). */
/* Outputs (device, caller-owned; n = number of points):                     */
/*   codes            uint32[n]  sorted unique Morton codes (first U valid)   */
/*   tree             arrays of >= n entries (first U - 1 valid)              */
/*   edge_count, prefix_sum  int32[n] (first U - 1 valid)                     */
/*   nodes            oct_node[nodes_capacity] (first M valid)                */
/*   d_counts         int32[4] = {U, U - 1, M, status bits}                   */
/* When M > nodes_capacity the octree stage is skipped and status carries    */
/* OCT_STATUS_CAPACITY; d_counts[2] still reports the M needed.              */
/* ----------------------------------------------------------------------- */
typedef struct oct_build_outputs {
  uint32_t* codes;
  oct_radix_tree tree;
  int32_t* edge_count;
  int32_t* prefix_sum;
  oct_node* nodes;
  int32_t nodes_capacity;
  int32_t* d_counts;
} oct_build_outputs;

OCT_API size_t oct_build_workspace_bytes(int n, int nodes_capacity);
OCT_API int oct_build_octree(const oct_vec4* points, int n, float min_coord, float range,
                     const oct_build_outputs* out, void* workspace, size_t workspace_bytes,
                     oct_stream_t stream);

/* Which form stages 2-3 took in the last whole build of n points with this
 * workspace (read back after that build has finished): 0 the LSD radix passes
 * and run-head unique (clouds below 2^22 points), 1 the MSD form (top-digit
 * scatter, per-bucket bitmaps, pack), 2 the LSD form chosen by the device
 * because the top-digit buckets were too uneven. Both give the same bytes. */
#define OCT_SORT_FORM_LSD 0
#define OCT_SORT_FORM_MSD 1
#define OCT_SORT_FORM_LSD_FALLBACK 2
OCT_API int oct_build_sort_form(const void* workspace, int n, int nodes_capacity, int* form);

/* Timed build for measurement: the same launches as oct_build_octree, with
 * caller-created CUDA events (cudaEvent_t, passed as void*) recorded on the
 * stream at each step boundary: events[k] after step k of
 * oct_build_step_name(k) for k < oct_build_step_count() (step 0 is the start).
 * Bench tooling derives per-kernel device times from consecutive events. */
OCT_API int oct_build_step_count(void);
OCT_API const char* oct_build_step_name(int k);
OCT_API int oct_build_octree_timed(const oct_vec4* points, int n, float min_coord, float range,
                                   const oct_build_outputs* out, void* workspace,
                                   size_t workspace_bytes, void* const* events, int n_events,
                                   oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Learned CDF of the Morton-key distribution (the learned-sort extension;   */
/* no counterpart in the reference). A model lives in one device buffer: a   */
/* 256-byte versioned header plus arrays laid out for max_segments (<= 4096);*/
/* copying the buffer persists the model. Model: monotone piecewise-linear   */
/* CDF, knots at evenly spaced ranks of a sorted key sample, heights         */
/* y_k = cumsum(softplus(theta)) / sum(softplus(theta)), trained by Adam on  */
/* the mean squared error against the sample's empirical CDF. Bucket ids     */
/* come from exact fixed-point tables and never decrease with the key.       */
/* ----------------------------------------------------------------------- */
#define OCT_LCDF_MAX_SEGMENTS 4096
#define OCT_LCDF_MAX_BUCKETS 65536
/* Byte offsets of the model's parts: {x, theta, adam_m, adam_v, y, grad, yq,
 * slope, lut, bounds, blut, total}; x is uint32[K+1], theta/adam/y/grad float,
 * yq uint32[K+1], slope uint64[K], lut uint16[4097] (knots below each 2^18-key
 * cell), bounds uint32[NB+1] (smallest key of each bucket, 2^30 past the
 * last), blut uint16[16385] (bucket at the start of each 2^16-key cell). */
OCT_API int oct_lcdf_layout(int max_segments, size_t offsets[12]);
OCT_API size_t oct_lcdf_fit_workspace_bytes(int n_sample);
/* Sorts the sample into the workspace, places knots, runs `steps` Adam steps
 * (learning rate lr) and builds bucket tables for n_buckets (<= 65536). */
OCT_API int oct_lcdf_fit(const uint32_t* sample_keys, int n_sample, int n_segments, int steps,
                         float lr, int n_buckets, void* model, int max_segments,
                         void* workspace, size_t workspace_bytes, oct_stream_t stream);
/* Loss (written into the header) and dL/dtheta (d_grad, K floats) of the
 * model's current theta on a SORTED sample. */
OCT_API int oct_lcdf_loss_grad(const uint32_t* sorted_sample, int n_sample, void* model,
                               int max_segments, float* d_grad, oct_stream_t stream);
/* `steps` more Adam steps (learning rate lr) on the model's current theta. */
OCT_API int oct_lcdf_train_steps(const uint32_t* sorted_sample, int n_sample, void* model,
                                 int max_segments, int steps, float lr, oct_stream_t stream);
/* Rebuild the bucket tables from the current theta for n_buckets. */
OCT_API int oct_lcdf_tables(void* model, int max_segments, int n_buckets, oct_stream_t stream);
/* d_buckets[i] = bucket of keys[i] (30-bit keys). */
OCT_API int oct_lcdf_buckets(const void* model, int max_segments, const uint32_t* keys, int n,
                             uint32_t* d_buckets, oct_stream_t stream);

/* Learned bucketed sort + unique: sorted unique keys of keys[0, n) (30-bit)
 * into out_unique and U into *d_n_unique, through `model` (tables built for
 * n_buckets). Keys are scattered into model buckets and each bucket is sorted
 * and de-duplicated in shared memory; when more than overflow_threshold of the
 * keys sit in oversized buckets, or a bucket fits no shared-memory form, the
 * same launches fall back to the OneSweep sort + unique (device-side switch).
 * d_stats (nullable, 48 bytes): {fallback, failed_buckets, overflow_keys,
 * max_bucket, n, overflow_frac (float), skip, bitmap_buckets, radix_buckets,
 * bitonic_buckets, 0, 0}. On the fallback path `keys`
 * is sorted in place; otherwise it is left as it was. */
OCT_API size_t oct_lsort_workspace_bytes(int n, int n_buckets, int max_segments);
OCT_API int oct_lsort_unique(uint32_t* keys, int n, const void* model, int max_segments,
                             int n_buckets, float overflow_threshold, uint32_t* out_unique,
                             int32_t* d_n_unique, void* d_stats, void* workspace,
                             size_t workspace_bytes, uint32_t* d_status, oct_stream_t stream);
/* Whole build with the learned sort for stages 2-3 (outputs as oct_build_octree). */
OCT_API size_t oct_build_learned_workspace_bytes(int n, int nodes_capacity, int n_buckets,
                                                 int max_segments);
OCT_API int oct_build_octree_learned(const oct_vec4* points, int n, float min_coord, float range,
                                     const void* model, int max_segments, int n_buckets,
                                     float overflow_threshold, const oct_build_outputs* out,
                                     void* d_stats, void* workspace, size_t workspace_bytes,
                                     oct_stream_t stream);
/* Radix sort shape used by sort plans made after the call (the autotuner's
 * knob): radix_bits 10 or 8, warps 16, items 16 or 24, scan 0 (decoupled
 * look-back) or 1 (per-tile histograms + tile scan). */
OCT_API int oct_set_sort_config(int radix_bits, int warps, int items, int scan);
OCT_API int oct_get_sort_config(int out[4]);

/* ----------------------------------------------------------------------- */
/* Batched build: many clouds of uneven size in one launch sequence (the     */
/* batched-build extension; no counterpart in the reference, whose drivers   */
/* build one cloud per run). Points of all clouds are concatenated; cloud c  */
/* owns points / codes / tree arrays / edge counts / prefix sums at          */
/* [start_c, start_c + n_c) and OctNodes at [node_start_c, node_start_c +    */
/* cap_c). Each cloud's outputs are bit-identical to oct_build_octree on it. */
/* The plan (a host object) fixes the cloud sizes and the sort shape; its    */
/* device tables are uploaded once; builds are capturable in CUDA graphs.    */
/* d_cloud_counts: int32[4 * n_clouds] = per cloud {U, U-1, M, status}.     */
/* ----------------------------------------------------------------------- */
typedef struct oct_batch_plan oct_batch_plan;
/* h_node_caps may be NULL (cap_c = n_c). Returns NULL on bad sizes. */
OCT_API oct_batch_plan* oct_batch_plan_create(int n_clouds, const int32_t* h_cloud_sizes,
                                              const int32_t* h_node_caps);
OCT_API void oct_batch_plan_destroy(oct_batch_plan* plan);
/* {n_clouds, total points, total OctNode capacity, table bytes, workspace
 * bytes, sort tiles} */
OCT_API int oct_batch_plan_info(const oct_batch_plan* plan, int64_t out[6]);
/* Copies the plan's tables into d_tables (256-byte aligned, table bytes). */
OCT_API int oct_batch_upload_tables(const oct_batch_plan* plan, void* d_tables,
                                    oct_stream_t stream);
OCT_API int oct_build_octree_batch(const oct_batch_plan* plan, const void* d_tables,
                                   const oct_vec4* points, const float* d_mins,
                                   const float* d_ranges, const oct_build_outputs* out,
                                   int32_t* d_cloud_counts, void* workspace,
                                   size_t workspace_bytes, oct_stream_t stream);

/* Scheduling of the batched build's octree-stage kernels (prefix sum, emit,
 * finalize): 1 persistent CTAs take their tiles from an atomic work queue;
 * 0 (default) one CTA per tile by block index (the tiles are of equal size:
 * the queue measured 0.99x on the 512-cloud batch). Results are the same.
 * Applies to later builds in this process. */
OCT_API int oct_set_batch_work_queue(int on);

/* Learned + batched build (no counterpart in the reference): the batched
 * build with stage 2 done by one learned CDF model shared by the clouds
 * (fit on their own per-cloud Morton codes, oct_lcdf_fit): per cloud, each
 * key goes to one of n_buckets buckets, each bucket is sorted in shared
 * memory down to its unique keys (a bitmap over the bucket's key span, or a
 * radix or bitonic sort). When a bucket fits none of those forms the plain
 * LSD passes sort the batch instead (decided on the device). Outputs are the
 * batched build's, bit for bit. d_stats (may be NULL): 12 words, as
 * oct_build_octree_learned's (word 0: 1 if the LSD passes ran; word 3: the
 * largest bucket; words 7-9: buckets done by bitmap, radix and bitonic sort).
 * Workspace: oct_batch_learned_workspace_bytes(plan, n_buckets).
 * Needs a sort shape with an odd pass count (the default: 3 x 10 bits). */
OCT_API size_t oct_batch_learned_workspace_bytes(const oct_batch_plan* plan, int n_buckets);
OCT_API int oct_build_octree_batch_learned(const oct_batch_plan* plan, const void* d_tables,
                                           const oct_vec4* points, const float* d_mins,
                                           const float* d_ranges, const void* model,
                                           int max_segments, int n_buckets,
                                           const oct_build_outputs* out, int32_t* d_cloud_counts,
                                           uint32_t* d_stats, void* workspace,
                                           size_t workspace_bytes, oct_stream_t stream);

/* Synchronous convenience: copies d_counts to the host after the stream
 * drains and maps the status word to OCT_ERR_DEVICE / OCT_ERR_CAPACITY. */
OCT_API int oct_read_counts(const int32_t* d_counts, int32_t* h_counts, oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Octree consumers: Morton decode and the tree check.                      */
/* oct_morton_decode: d_out[i] = morton32_to_xyz(codes[i]) (include/shared/ */
/* morton.h:45-80): per axis (raw / 1024) * range + min in FP32 without      */
/* contraction, w = 1. d_out 16-byte aligned.                                */
/* oct_check_tree: checkTree (apps/cpu_demo/main.cpp:13-35) from node        */
/* root_index with (root_prefix, root_code_len): child_node_mask bits        */
/* descend to children[c] with prefix << 3 | c and code length + 3;          */
/* child_leaf_mask bits compare codes[children[c]] >> (30 - length - 3) with  */
/* that prefix. d_counts (4 x int64, device) = {nodes visited, leaf checks,   */
/* mismatches, rejected}; rejected counts steps the reference would take out */
/* of bounds (child index outside the arrays, code length past 30) and, on a */
/* malformed tree, visits beyond n_nodes per level. No counterpart runs in    */
/* the reference's drivers (the function is defined but not called).         */
/* ----------------------------------------------------------------------- */
OCT_API int oct_morton_decode(const uint32_t* codes, int n, float min_coord, float range,
                              oct_vec4* d_out, oct_stream_t stream);
OCT_API size_t oct_check_tree_workspace_bytes(int n_nodes);
OCT_API int oct_check_tree(const oct_node* nodes, int n_nodes, const uint32_t* codes, int n_codes,
                           uint32_t root_prefix, int root_code_len, int root_index,
                           long long* d_counts, void* workspace, size_t workspace_bytes,
                           oct_stream_t stream);

/* ----------------------------------------------------------------------- */
/* Diagnostics: bounded look-back waits. No counterpart in the reference,    */
/* whose look-back spins have no bound (kernels/cuda/02_sort.cu:461-479).    */
/* Every look-back wait of this library gives up after 1 s without its flag, */
/* sets OCT_STATUS_SPIN_TIMEOUT in the status word and lets its kernel       */
/* return. This call runs one such wait on a tile whose predecessor never    */
/* publishes (the workspace is cleared first), with the bound limit_ns (at   */
/* most 1 s), so a caller can check that it returns within that time with   */
/* the bit set. which: OCT_DIAG_WAIT_SORT (the sort's per-digit look-back)   */
/* or OCT_DIAG_WAIT_SCAN (the warp look-back of unique and prefix sum).      */
/* workspace: DEVICE, 256-byte aligned, oct_diag_wait_workspace_bytes().     */
/* ----------------------------------------------------------------------- */
#define OCT_DIAG_WAIT_SORT 0
#define OCT_DIAG_WAIT_SCAN 1
OCT_API size_t oct_diag_wait_workspace_bytes(void);
OCT_API int oct_diag_lookback_timeout(int which, unsigned long long limit_ns, void* workspace,
                                      size_t workspace_bytes, uint32_t* d_status,
                                      oct_stream_t stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* OCTREE_GB300_H */
