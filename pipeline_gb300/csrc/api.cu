// C ABI of libpipeline_gb300.so (declared in include/octree_gb300.h).
//
// Host-side only: validates arguments, carves caller workspaces, launches the
// stage kernels on the caller's stream. No call allocates device memory.
#include <stdio.h>
#include <string.h>

#include "kernels.cuh"

using namespace octgb;

namespace {

thread_local char g_last_error[256] = "";

int cuda_fail(cudaError_t e, const char* where) {
  snprintf(g_last_error, sizeof(g_last_error), "%s: %s", where, cudaGetErrorString(e));
  return OCT_ERR_CUDA;
}

#define OCT_TRY(expr, where)                      \
  do {                                            \
    cudaError_t e_ = (expr);                      \
    if (e_ != cudaSuccess) return cuda_fail(e_, where); \
  } while (0)

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

cudaStream_t S(oct_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// Control block shared by the whole build: zeroed by one memset per build.
struct BuildLayout {
  SortPlan sort;
  ScanPlan uniq;
  size_t sort_off, uniq_off, misc_off, ctrl_bytes;
  size_t msd_off, keys_a_off, keys_b_off, tree_off, tags_off, total;
};

BuildLayout build_layout(int n, int cap) {
  BuildLayout L{};
  L.sort = sort_plan(n, 30);
  L.uniq = unique_plan(n);
  // Everything that must start at zero is contiguous from offset 0 up to the
  // end of the sort's zeroed part; the sort's digit bases and per-tile
  // histograms (always fully written before use) follow.
  L.uniq_off = 0;
  L.misc_off = align_up(L.uniq_off + L.uniq.bytes, 256);
  L.sort_off = align_up(L.misc_off + 256, 256);
  L.ctrl_bytes = L.sort_off + L.sort.zero_bytes;
  L.msd_off = align_up(L.sort_off + L.sort.bytes, 256);
  L.keys_a_off = align_up(L.msd_off + msd_scratch_bytes(), 256);
  L.keys_b_off = align_up(L.keys_a_off + sizeof(uint32_t) * (size_t)(n > 0 ? n : 1), 256);
  L.tree_off = align_up(L.keys_b_off + sizeof(uint32_t) * (size_t)(n > 0 ? n : 1), 256);
  L.tags_off = align_up(L.tree_off + tree_scratch_bytes(n), 256);
  L.total = align_up(L.tags_off + oct_tags_bytes(cap), 256);
  return L;
}

// misc area: [0] status, [1] n_unique, [2] max octree slot, [4..5] sort form
// flags (MSD, LSD)
struct Misc {
  uint32_t* status;
  int* unique;
  int* max_slot;
  uint32_t* form;
};
Misc misc_at(char* base) {
  Misc m;
  m.status = reinterpret_cast<uint32_t*>(base);
  m.unique = reinterpret_cast<int*>(base + 4);
  m.max_slot = reinterpret_cast<int*>(base + 8);
  m.form = reinterpret_cast<uint32_t*>(base + 16);
  return m;
}

__global__ void node_count_init_kernel(const int* ps, int n, int* out) { *out = ps[n - 1]; }

__global__ void node_count_kernel(const int* __restrict__ ec, const int* __restrict__ ps, int n,
                                  int* out) {
  int mx = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (i > 0 && ec[i] > 0) mx = max(mx, ps[i] + ec[i] - 1);
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0 && mx > 0) atomicMax(out, mx);
}

__global__ void plus_one_kernel(int* v) { *v += 1; }

__global__ void root_init_kernel(oct_node* nodes, const uint32_t* codes, const uint8_t* prefix_n,
                                 float min_coord, float range) {
  const int root_level = prefix_n[0] / 3;
  const int sh = 30 - 3 * root_level;
  const float4 c = decode_corner((codes[0] >> sh) << sh, min_coord, range);
  nodes[0].corner.x = c.x;
  nodes[0].corner.y = c.y;
  nodes[0].corner.z = c.z;
  nodes[0].corner.w = c.w;
  nodes[0].cell_size = range;
}

}  // namespace

void octgb::set_last_error(const char* msg) {
  snprintf(g_last_error, sizeof(g_last_error), "%s", msg);
}

static_assert(sizeof(oct_node) == 60, "oct_node must match OctNode (60 bytes)");
static_assert(offsetof(oct_node, corner) == 32, "OctNode::corner at byte 32");
static_assert(offsetof(oct_node, cell_size) == 48, "OctNode::cell_size at byte 48");
static_assert(offsetof(oct_node, child_node_mask) == 52, "OctNode::child_node_mask at 52");
static_assert(offsetof(oct_node, child_leaf_mask) == 56, "OctNode::child_leaf_mask at 56");
static_assert(sizeof(oct_vec4) == 16, "oct_vec4 must match glm::vec4");

extern "C" {

int oct_version(void) { return 100; }

int oct_built_arch(void) {
#if defined(OCT_BUILT_ARCH)
  return OCT_BUILT_ARCH;
#else
  return 0;
#endif
}

const char* oct_last_error(void) { return g_last_error; }

// ---------------------------------------------------------------- stage 1 --
int oct_morton_encode(const oct_vec4* points, uint32_t* keys, int64_t n, float min_coord,
                      float range, uint32_t* d_status, oct_stream_t stream) {
  if (n < 0 || n > OCT_MAX_N) return OCT_ERR_INVALID_ARG;
  if (n == 0) return OCT_OK;
  if (!points || !keys || !aligned(points, 16)) return OCT_ERR_INVALID_ARG;
  OCT_TRY(launch_morton(reinterpret_cast<const float4*>(points), keys, n, min_coord, range,
                        nullptr, nullptr, d_status, S(stream)),
          "oct_morton_encode");
  return OCT_OK;
}

// ---------------------------------------------------------------- stage 2 --
size_t oct_sort_workspace_bytes(int n, int key_bits) {
  if (n < 0 || key_bits < 1 || key_bits > 32) return 0;
  return sort_plan(n, key_bits).bytes;
}

int oct_sort_keys(uint32_t* keys, uint32_t* keys_alt, int n, int key_bits, void* workspace,
                  size_t workspace_bytes, uint32_t* d_status, oct_stream_t stream) {
  if (n < 0 || n > OCT_MAX_N || key_bits < 1 || key_bits > 32) return OCT_ERR_INVALID_ARG;
  if (n <= 1) return OCT_OK;
  if (!keys || !keys_alt || !workspace || !aligned(workspace, 256)) return OCT_ERR_INVALID_ARG;
  const SortPlan p = sort_plan(n, key_bits);
  if (workspace_bytes < p.bytes) return OCT_ERR_WORKSPACE;
  cudaStream_t s = S(stream);
  OCT_TRY(cudaMemsetAsync(workspace, 0, p.zero_bytes, s), "oct_sort_keys: clear");
  OCT_TRY(launch_histogram(keys, &p, workspace, s), "oct_sort_keys: histogram");
  uint32_t* result = keys;
  OCT_TRY(launch_sort_passes(keys, keys_alt, &p, workspace, d_status, s, &result),
          "oct_sort_keys: passes");
  if (result != keys)
    OCT_TRY(cudaMemcpyAsync(keys, result, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s),
            "oct_sort_keys: copy back");
  return OCT_OK;
}

// ---------------------------------------------------------------- stage 3 --
size_t oct_unique_workspace_bytes(int n) { return n < 0 ? 0 : unique_plan(n).bytes; }

int oct_unique(uint32_t* keys, int n, int32_t* d_n_unique, void* workspace, size_t workspace_bytes,
               uint32_t* d_status, oct_stream_t stream) {
  if (n < 0 || n > OCT_MAX_N || !d_n_unique) return OCT_ERR_INVALID_ARG;
  cudaStream_t s = S(stream);
  if (n == 0) {
    OCT_TRY(cudaMemsetAsync(d_n_unique, 0, sizeof(int32_t), s), "oct_unique");
    return OCT_OK;
  }
  if (!keys || !workspace || !aligned(workspace, 256)) return OCT_ERR_INVALID_ARG;
  const ScanPlan p = unique_plan(n);
  if (workspace_bytes < p.bytes) return OCT_ERR_WORKSPACE;
  OCT_TRY(cudaMemsetAsync(workspace, 0, p.bytes, s), "oct_unique: clear");
  OCT_TRY(launch_unique(keys, keys, n, d_n_unique, &p, workspace, d_status, s), "oct_unique");
  return OCT_OK;
}

// ---------------------------------------------------------------- stage 4 --
int oct_build_radix_tree(int n_nodes, const uint32_t* codes, uint8_t* prefix_n,
                         uint8_t* has_leaf_left, uint8_t* has_leaf_right, int32_t* left_child,
                         int32_t* parent, oct_stream_t stream) {
  if (n_nodes < 0 || n_nodes > OCT_MAX_N - 1) return OCT_ERR_INVALID_ARG;
  if (n_nodes == 0) return OCT_OK;
  if (!codes || !prefix_n || !has_leaf_left || !has_leaf_right || !left_child || !parent)
    return OCT_ERR_INVALID_ARG;
  OCT_TRY(launch_radix_tree(n_nodes, nullptr, codes, prefix_n, has_leaf_left, has_leaf_right,
                            left_child, parent, S(stream)),
          "oct_build_radix_tree");
  return OCT_OK;
}

size_t oct_radix_tree_sorted_workspace_bytes(int n_nodes) {
  if (n_nodes < 0 || n_nodes > OCT_MAX_N - 1) return 0;
  return tree_scratch_bytes(n_nodes);
}

int oct_build_radix_tree_sorted(int n_nodes, const uint32_t* codes, uint8_t* prefix_n,
                                uint8_t* has_leaf_left, uint8_t* has_leaf_right,
                                int32_t* left_child, int32_t* parent, int32_t* edge_count,
                                void* workspace, size_t workspace_bytes, oct_stream_t stream) {
  if (n_nodes < 0 || n_nodes > OCT_MAX_N - 1) return OCT_ERR_INVALID_ARG;
  if (n_nodes == 0) return OCT_OK;
  if (!codes || !prefix_n || !has_leaf_left || !has_leaf_right || !left_child || !parent ||
      !workspace || !aligned(workspace, 256))
    return OCT_ERR_INVALID_ARG;
  if (workspace_bytes < tree_scratch_bytes(n_nodes)) return OCT_ERR_WORKSPACE;
  OCT_TRY(launch_radix_tree_sorted(n_nodes, nullptr, codes, prefix_n, has_leaf_left,
                                   has_leaf_right, left_child, parent, edge_count, workspace,
                                   S(stream)),
          "oct_build_radix_tree_sorted");
  return OCT_OK;
}

// ---------------------------------------------------------------- stage 5 --
int oct_edge_count(const uint8_t* prefix_n, const int32_t* parent, int32_t* edge_count,
                   int n_nodes, oct_stream_t stream) {
  if (n_nodes < 0 || n_nodes > OCT_MAX_N) return OCT_ERR_INVALID_ARG;
  if (n_nodes == 0) return OCT_OK;
  if (!prefix_n || !parent || !edge_count) return OCT_ERR_INVALID_ARG;
  const ScanPlan p = edge_scan_plan(n_nodes);
  OCT_TRY(launch_edge_scan(kEdgeOnly, n_nodes, nullptr, prefix_n, parent, edge_count, nullptr,
                           nullptr, &p, nullptr, nullptr, S(stream)),
          "oct_edge_count");
  return OCT_OK;
}

// ---------------------------------------------------------------- stage 6 --
size_t oct_prefix_sum_workspace_bytes(int n) { return n < 0 ? 0 : edge_scan_plan(n).bytes; }

int oct_prefix_sum(const int32_t* data, int n, int32_t* out, void* workspace,
                   size_t workspace_bytes, uint32_t* d_status, oct_stream_t stream) {
  if (n < 0 || n > OCT_MAX_N) return OCT_ERR_INVALID_ARG;
  if (n == 0) return OCT_OK;
  if (!data || !out || !workspace || !aligned(workspace, 256)) return OCT_ERR_INVALID_ARG;
  const ScanPlan p = edge_scan_plan(n);
  if (workspace_bytes < p.bytes) return OCT_ERR_WORKSPACE;
  cudaStream_t s = S(stream);
  OCT_TRY(cudaMemsetAsync(workspace, 0, p.bytes, s), "oct_prefix_sum: clear");
  OCT_TRY(launch_edge_scan(kScanOnly, n, nullptr, nullptr, nullptr, const_cast<int*>(data), out,
                           nullptr, &p, workspace, d_status, s),
          "oct_prefix_sum");
  return OCT_OK;
}

int oct_octree_node_count(const int32_t* edge_count, const int32_t* prefix_sum, int n_nodes,
                          int32_t* d_n_oct_nodes, oct_stream_t stream) {
  if (n_nodes < 0 || !d_n_oct_nodes) return OCT_ERR_INVALID_ARG;
  cudaStream_t s = S(stream);
  if (n_nodes == 0) {
    OCT_TRY(cudaMemsetAsync(d_n_oct_nodes, 0, sizeof(int32_t), s), "oct_octree_node_count");
    return OCT_OK;
  }
  if (!edge_count || !prefix_sum) return OCT_ERR_INVALID_ARG;
  node_count_init_kernel<<<1, 1, 0, s>>>(prefix_sum, n_nodes, d_n_oct_nodes);
  int grid = (n_nodes + 255) / 256;
  if (grid > device_sm_count() * 8) grid = device_sm_count() * 8;
  node_count_kernel<<<grid, 256, 0, s>>>(edge_count, prefix_sum, n_nodes, d_n_oct_nodes);
  plus_one_kernel<<<1, 1, 0, s>>>(d_n_oct_nodes);
  OCT_TRY(cudaGetLastError(), "oct_octree_node_count");
  return OCT_OK;
}

// ------------------------------------------------------------ stages 7-8 --
size_t oct_octree_workspace_bytes(int n_oct_nodes) {
  return n_oct_nodes < 0 ? 0 : oct_tags_bytes(n_oct_nodes);
}

int oct_octree_root_init(oct_node* nodes, const uint32_t* codes, const uint8_t* prefix_n,
                         float min_coord, float range, oct_stream_t stream) {
  if (!nodes || !codes || !prefix_n) return OCT_ERR_INVALID_ARG;
  root_init_kernel<<<1, 1, 0, S(stream)>>>(nodes, codes, prefix_n, min_coord, range);
  OCT_TRY(cudaGetLastError(), "oct_octree_root_init");
  return OCT_OK;
}

static int octree_stage(int mode, oct_node* nodes, int n_oct_nodes, const int32_t* offsets,
                        const int32_t* counts, const uint32_t* codes, const uint8_t* hll,
                        const uint8_t* hlr, const uint8_t* prefix_n, const int32_t* parents,
                        const int32_t* left_child, float min_coord, float range, int n_nodes,
                        void* workspace, size_t workspace_bytes, uint32_t* d_status,
                        oct_stream_t stream) {
  if (n_nodes < 0 || n_oct_nodes < 0 || n_nodes > OCT_MAX_N || n_oct_nodes > OCT_MAX_N)
    return OCT_ERR_INVALID_ARG;
  if (n_nodes > OCT_MAX_OCTREE_NODES) return OCT_ERR_TOO_LARGE;
  if (n_nodes == 0 || n_oct_nodes == 0) return OCT_OK;
  if (!nodes || !offsets || !counts || !codes || !prefix_n || !parents || !workspace ||
      !aligned(workspace, 256))
    return OCT_ERR_INVALID_ARG;
  if ((mode & kOctLink) && (!hll || !hlr || !left_child)) return OCT_ERR_INVALID_ARG;
  if (workspace_bytes < oct_tags_bytes(n_oct_nodes)) return OCT_ERR_WORKSPACE;
  OctArgs a{};
  a.nodes = nodes;
  a.cap = n_oct_nodes;
  a.offsets = offsets;
  a.counts = counts;
  a.codes = codes;
  a.prefix_n = prefix_n;
  a.hll = hll;
  a.hlr = hlr;
  a.parent = parents;
  a.left_child = left_child;
  a.min_coord = min_coord;
  a.range = range;
  a.n_brt_host = n_nodes;
  a.n_oct_host = n_oct_nodes;
  const OctTags t = oct_tags_carve(workspace, n_oct_nodes);
  OCT_TRY(launch_octree(mode, a, t, d_status, S(stream)), "octree stage");
  return OCT_OK;
}

int oct_make_oct_nodes(oct_node* nodes, int n_oct_nodes, const int32_t* node_offsets,
                       const int32_t* rt_node_counts, const uint32_t* codes,
                       const uint8_t* rt_prefix_n, const int32_t* rt_parents, float min_coord,
                       float range, int n_nodes, void* workspace, size_t workspace_bytes,
                       uint32_t* d_status, oct_stream_t stream) {
  return octree_stage(kOctMake, nodes, n_oct_nodes, node_offsets, rt_node_counts, codes, nullptr,
                      nullptr, rt_prefix_n, rt_parents, nullptr, min_coord, range, n_nodes,
                      workspace, workspace_bytes, d_status, stream);
}

int oct_link_leaf_nodes(oct_node* nodes, int n_oct_nodes, const int32_t* node_offsets,
                        const int32_t* rt_node_counts, const uint32_t* codes,
                        const uint8_t* rt_has_leaf_left, const uint8_t* rt_has_leaf_right,
                        const uint8_t* rt_prefix_n, const int32_t* rt_parents,
                        const int32_t* rt_left_child, int n_nodes, void* workspace,
                        size_t workspace_bytes, uint32_t* d_status, oct_stream_t stream) {
  return octree_stage(kOctLink, nodes, n_oct_nodes, node_offsets, rt_node_counts, codes,
                      rt_has_leaf_left, rt_has_leaf_right, rt_prefix_n, rt_parents, rt_left_child,
                      0.f, 1.f, n_nodes, workspace, workspace_bytes, d_status, stream);
}

// ------------------------------------------------------------ whole build --
size_t oct_build_workspace_bytes(int n, int nodes_capacity) {
  if (n < 0 || nodes_capacity < 0) return 0;
  return build_layout(n, nodes_capacity).total;
}

static int build_impl(const oct_vec4* points, int n, float min_coord, float range,
                      const oct_build_outputs* out, void* workspace, size_t workspace_bytes,
                      oct_stream_t stream, Recorder* rec) {
  if (n < 0 || n > OCT_MAX_N || !out || !out->d_counts) return OCT_ERR_INVALID_ARG;
  if (out->nodes_capacity > 0 && n > OCT_MAX_OCTREE_NODES + 1) return OCT_ERR_TOO_LARGE;
  cudaStream_t s = S(stream);
  if (n == 0) {
    OCT_TRY(cudaMemsetAsync(out->d_counts, 0, 4 * sizeof(int32_t), s), "oct_build_octree");
    return OCT_OK;
  }
  if (!points || !aligned(points, 16) || !out->codes || !out->tree.prefix_n ||
      !out->tree.has_leaf_left || !out->tree.has_leaf_right || !out->tree.left_child ||
      !out->tree.parent || !out->edge_count || !out->prefix_sum ||
      (out->nodes_capacity > 0 && !out->nodes) || out->nodes_capacity < 0 || !workspace ||
      !aligned(workspace, 256))
    return OCT_ERR_INVALID_ARG;
  const BuildLayout L = build_layout(n, out->nodes_capacity);
  if (workspace_bytes < L.total) return OCT_ERR_WORKSPACE;
  char* w = static_cast<char*>(workspace);
  const Misc m = misc_at(w + L.misc_off);
  uint32_t* keys_a = reinterpret_cast<uint32_t*>(w + L.keys_a_off);
  uint32_t* keys_b = reinterpret_cast<uint32_t*>(w + L.keys_b_off);

  mark(rec, s);
  OCT_TRY(cudaMemsetAsync(w, 0, L.ctrl_bytes, s), "build: clear");
  mark(rec, s);
  OCT_TRY(launch_morton(reinterpret_cast<const float4*>(points), keys_a, n, min_coord, range,
                        &L.sort, w + L.sort_off, m.status, s),
          "build: morton");
  mark(rec, s);
  // Stages 2-3: LSD passes + run-head unique, or for large even clouds the
  // MSD form (top-digit scatter, per-bucket bitmaps, pack), chosen on the
  // device from the top-digit histogram; both write the sorted unique codes,
  // U and the deltas of adjacent codes, from which the tree (with the edge
  // counts) is built.
  const bool msd = n >= msd_min_n() && msd_plan_ok(L.sort);
  char* sort_ctrl = w + L.sort_off;
  const uint32_t* top_hist = reinterpret_cast<const uint32_t*>(sort_ctrl + L.sort.hist_off) +
                             (size_t)(L.sort.passes - 1) * L.sort.bins;
  const uint32_t* top_base = reinterpret_cast<const uint32_t*>(sort_ctrl + L.sort.base_off) +
                             (size_t)(L.sort.passes - 1) * L.sort.bins;
  if (msd) OCT_TRY(launch_msd_gate(top_hist, n, m.form, s), "build: sort form");
  uint32_t* sorted = keys_a;
  OCT_TRY(launch_sort_passes_split(keys_a, keys_b, &L.sort, sort_ctrl, m.status,
                                   msd ? m.form : nullptr, msd ? m.form + 1 : nullptr, s, &sorted,
                                   rec),
          "build: sort");
  if (msd) {
    OCT_TRY(launch_msd_buckets(keys_b, top_base, top_hist, w + L.msd_off, m.form, m.status, s),
            "build: msd buckets");
  }
  mark(rec, s);
  OCT_TRY(launch_unique_deltas(sorted, n, out->codes, m.unique, w + L.tree_off, s,
                               msd ? m.form + 1 : nullptr),
          "build: unique");
  if (msd) {
    OCT_TRY(launch_msd_pack(keys_b, top_base, n, out->codes, m.unique, w + L.msd_off,
                            w + L.tree_off, m.form, s),
            "build: msd pack");
  }
  mark(rec, s);
  OCT_TRY(launch_radix_tree_from_deltas(n, m.unique, out->codes, out->tree.prefix_n,
                                        out->tree.has_leaf_left, out->tree.has_leaf_right,
                                        out->tree.left_child, out->tree.parent, out->edge_count,
                                        w + L.tree_off, s),
          "build: radix tree");
  mark(rec, s);
  const OctTags tags = oct_tags_carve(w + L.tags_off, out->nodes_capacity);
  OCT_TRY(launch_prefix_sum_clear_tags(n, m.unique, out->edge_count, out->prefix_sum, m.max_slot,
                                       w + L.tree_off, m.status, tags, s),
          "build: prefix sum");
  mark(rec, s);
  if (out->nodes_capacity > 0) {
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
    a.d_unique = m.unique;
    a.d_max_slot = m.max_slot;
    OCT_TRY(launch_octree(kOctMake | kOctLink | kOctFresh, a, tags, m.status, s, rec, true),
            "build: octree");
  } else {
    for (int k = 0; k < 2; ++k) mark(rec, s);
  }
  OCT_TRY(launch_publish_counts(m.unique, m.max_slot, m.status, out->d_counts, s),
          "build: counts");
  mark(rec, s);
  return OCT_OK;
}

int oct_build_octree(const oct_vec4* points, int n, float min_coord, float range,
                     const oct_build_outputs* out, void* workspace, size_t workspace_bytes,
                     oct_stream_t stream) {
  return build_impl(points, n, min_coord, range, out, workspace, workspace_bytes, stream,
                    nullptr);
}

static const char* const kBuildSteps[] = {
    "start",       "clear",       "morton+histogram", "histogram scan",
    "sort pass 0", "sort pass 1", "sort pass 2",      "msd buckets",
    "unique",      "radix tree+edge count", "prefix sum", "octree emit",
    "octree finalize", "publish counts"};

int oct_build_sort_form(const void* workspace, int n, int nodes_capacity, int* form) {
  if (!workspace || !form || n < 0 || n > OCT_MAX_N || nodes_capacity < 0)
    return OCT_ERR_INVALID_ARG;
  const BuildLayout L = build_layout(n, nodes_capacity);
  if (n < msd_min_n() || !msd_plan_ok(L.sort)) {
    *form = OCT_SORT_FORM_LSD;
    return OCT_OK;
  }
  uint32_t f[2] = {0, 0};
  OCT_TRY(cudaMemcpy(f, static_cast<const char*>(workspace) + L.misc_off + 16, sizeof(f),
                     cudaMemcpyDeviceToHost),
          "oct_build_sort_form");
  *form = f[0] ? OCT_SORT_FORM_MSD : OCT_SORT_FORM_LSD_FALLBACK;
  return OCT_OK;
}

int oct_build_step_count(void) { return (int)(sizeof(kBuildSteps) / sizeof(kBuildSteps[0])); }

const char* oct_build_step_name(int k) {
  return (k >= 0 && k < oct_build_step_count()) ? kBuildSteps[k] : "";
}

int oct_build_octree_timed(const oct_vec4* points, int n, float min_coord, float range,
                           const oct_build_outputs* out, void* workspace, size_t workspace_bytes,
                           void* const* events, int n_events, oct_stream_t stream) {
  if (n_events < 0 || (n_events > 0 && !events)) return OCT_ERR_INVALID_ARG;
  Recorder r;
  r.events = reinterpret_cast<cudaEvent_t*>(const_cast<void**>(events));
  r.n = n_events;
  const int rc = build_impl(points, n, min_coord, range, out, workspace, workspace_bytes, stream, &r);
  if (rc == OCT_OK && r.err != cudaSuccess) {
    cudaGetLastError();
    return cuda_fail(r.err, "oct_build_octree_timed: event record");
  }
  return rc;
}



size_t oct_diag_wait_workspace_bytes(void) { return 2 * 1024 * sizeof(uint32_t); }

int oct_diag_lookback_timeout(int which, unsigned long long limit_ns, void* workspace,
                              size_t workspace_bytes, uint32_t* d_status, oct_stream_t stream) {
  if ((which != OCT_DIAG_WAIT_SORT && which != OCT_DIAG_WAIT_SCAN) || limit_ns == 0 ||
      limit_ns > kWaitLimitNs || !workspace || !aligned(workspace, 256) || !d_status)
    return OCT_ERR_INVALID_ARG;
  if (workspace_bytes < oct_diag_wait_workspace_bytes()) return OCT_ERR_WORKSPACE;
  cudaStream_t s = S(stream);
  // Every look-back word starts unpublished; nothing publishes tile 0.
  OCT_TRY(cudaMemsetAsync(workspace, 0, oct_diag_wait_workspace_bytes(), s), "oct_diag: clear");
  if (which == OCT_DIAG_WAIT_SORT)
    OCT_TRY(launch_diag_sort_wait(static_cast<uint32_t*>(workspace), d_status, limit_ns, s),
            "oct_diag_lookback_timeout");
  else
    OCT_TRY(launch_diag_scan_wait(static_cast<unsigned long long*>(workspace), d_status, limit_ns,
                                  s),
            "oct_diag_lookback_timeout");
  return OCT_OK;
}

int oct_read_counts(const int32_t* d_counts, int32_t* h_counts, oct_stream_t stream) {
  if (!d_counts || !h_counts) return OCT_ERR_INVALID_ARG;
  cudaStream_t s = S(stream);
  OCT_TRY(cudaMemcpyAsync(h_counts, d_counts, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, s),
          "oct_read_counts");
  OCT_TRY(cudaStreamSynchronize(s), "oct_read_counts: sync");
  const uint32_t st = (uint32_t)h_counts[3];
  if (st & OCT_STATUS_CAPACITY) return OCT_ERR_CAPACITY;
  if (st) return OCT_ERR_DEVICE;
  return OCT_OK;
}

}  // extern "C"
