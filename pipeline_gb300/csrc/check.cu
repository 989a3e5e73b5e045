// Device-side input generator, Morton decode and octree check.
//
//   oct_init_random_vec4_device  the reference's device generator
//       (kernels/cuda/00_init.cu:11-50) element by element, as its driver
//       launches it (apps/gpu_demo/main.cu:168-175: one element per thread,
//       so element i's four states are seeded from 4i .. 4i+3); any grid here
//       gives the same array
//   oct_morton_decode            morton32_to_xyz (include/shared/morton.h:45-80)
//   oct_check_tree               checkTree (apps/cpu_demo/main.cpp:13-35) as a
//       level-synchronous traversal: one launch per 3-bit level, the frontier
//       of (node, prefix, code length) in a workspace queue
#include "kernels.cuh"

namespace octgb {

// --------------------------------------------------------------- generator --
// Hybrid Tausworthe/LCG generator (GPU Gems 3 ch. 37): one step of three
// Tausworthe generators and one LCG from the seeded states; u = low 24 bits
// / 2^24, value = min + u * range as one fused multiply-add (nvcc's default
// contraction of the reference's expression).
__device__ __forceinline__ float gen_value(uint32_t v, float min_coord, float range) {
  const float u = __fmul_rn(__uint2float_rn(v & 0xFFFFFFu), 0x1p-24f);
  return __fmaf_rn(u, range, min_coord);
}

__global__ void __launch_bounds__(256)
    init_random_vec4_kernel(float4* __restrict__ out, int n, float min_coord, float range,
                            uint32_t seed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t b = (uint32_t)i << 2;
    uint32_t z1 = b * seed, z2 = (b + 1u) * seed, z3 = (b + 2u) * seed, z4 = (b + 3u) * seed;
    z1 = ((z1 & 4294967294u) << 12) ^ (((z1 << 13) ^ z1) >> 19);
    z2 = ((z2 & 4294967288u) << 4) ^ (((z2 << 2) ^ z2) >> 25);
    z3 = ((z3 & 4294967280u) << 17) ^ (((z3 << 3) ^ z3) >> 11);
    z4 = z4 * 1664525u + 1013904223u;
    out[i] = make_float4(gen_value(z1 ^ z2, min_coord, range), gen_value(z2 ^ z3, min_coord, range),
                         gen_value(z3 ^ z4, min_coord, range), gen_value(z1 ^ z4, min_coord, range));
  }
}

// Key sequences of kernels/00_init.cpp:5-17: keys[i] = n - i (descending) or
// i (ascending), as unsigned 32-bit values.
__global__ void __launch_bounds__(256)
    init_sequence_kernel(uint32_t* __restrict__ keys, int n, int descending) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    keys[i] = descending ? (uint32_t)(n - i) : (uint32_t)i;
}

// ------------------------------------------------------------------ decode --
__global__ void __launch_bounds__(256)
    morton_decode_kernel(const uint32_t* __restrict__ codes, int n, float min_coord, float range,
                         float4* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = decode_corner(codes[i], min_coord, range);
}

// ------------------------------------------------------------------- check --
// counts: {nodes visited, leaf checks, mismatches, rejected}. A rejected step
// is a child index outside the arrays, a level past 30 bits, or a visit that
// does not fit the frontier queue (capacity: the node count).
constexpr int kMortonBits = 30;

__global__ void __launch_bounds__(256)
    check_level_kernel(const oct_node* __restrict__ nodes, int n_nodes,
                       const uint32_t* __restrict__ codes, int n_codes,
                       const int4* __restrict__ in, const uint32_t* __restrict__ in_count,
                       int4* __restrict__ out, uint32_t* __restrict__ out_count, uint32_t cap,
                       unsigned long long* __restrict__ counts) {
  const uint32_t m = min(*in_count, cap);
  unsigned long long visited = 0, checks = 0, bad = 0, rejected = 0;
  const int lane = threadIdx.x & 31;
  for (uint32_t k0 = blockIdx.x * blockDim.x; k0 < m; k0 += gridDim.x * blockDim.x) {
    const uint32_t k = k0 + threadIdx.x;
    int node = 0, len = 0, nmask = 0, lmask = 0;
    uint32_t prefix = 0;
    const oct_node* nd = nullptr;
    if (k < m) {
      const int4 v = in[k];
      node = v.x;
      prefix = (uint32_t)v.y;
      len = v.z;
      nd = nodes + node;
      nmask = nd->child_node_mask & 0xff;
      lmask = nd->child_leaf_mask & 0xff;
      ++visited;
    }
    // children to visit next: valid index and depth
    uint32_t push = 0;
    int kids[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      kids[c] = 0;
      if (nmask & (1 << c)) {
        kids[c] = nd->children[c];
        if ((unsigned)kids[c] < (unsigned)n_nodes && len + 3 <= kMortonBits) push |= 1u << c;
        else ++rejected;
      }
    }
    // one queue reservation per warp
    const uint32_t cnt = __popc(push);
    uint32_t inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(out_count, total);
    base = __shfl_sync(0xffffffffu, base, 31) + inc - cnt;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (push & (1u << c)) {
        if (base < cap) out[base] = make_int4(kids[c], (int)((prefix << 3) | (uint32_t)c), len + 3, 0);
        else ++rejected;
        ++base;
      }
    }
    if (k < m && lmask) {
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        if (!(lmask & (1 << c))) continue;
        const int leaf = nd->children[c];
        if ((unsigned)leaf >= (unsigned)n_codes || len + 3 > kMortonBits) {
          ++rejected;
          continue;
        }
        ++checks;
        const uint32_t np = (prefix << 3) | (uint32_t)c;
        if ((codes[leaf] >> (kMortonBits - (len + 3))) != np) ++bad;
      }
    }
  }
  // warp sums, then one atomic per warp and counter
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    visited += __shfl_xor_sync(0xffffffffu, visited, o);
    checks += __shfl_xor_sync(0xffffffffu, checks, o);
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
    rejected += __shfl_xor_sync(0xffffffffu, rejected, o);
  }
  if (lane == 0) {
    if (visited) atomicAdd(counts + 0, visited);
    if (checks) atomicAdd(counts + 1, checks);
    if (bad) atomicAdd(counts + 2, bad);
    if (rejected) atomicAdd(counts + 3, rejected);
  }
}

__global__ void check_seed_kernel(int4* q, uint32_t* q_count, uint32_t* next_counts, int levels,
                                  int root, uint32_t prefix, int code_len, int n_nodes,
                                  unsigned long long* counts) {
  counts[0] = counts[1] = counts[2] = counts[3] = 0;
  for (int l = 0; l < levels; ++l) next_counts[l] = 0;
  if ((unsigned)root < (unsigned)n_nodes) {
    q[0] = make_int4(root, (int)prefix, code_len, 0);
    *q_count = 1;
  } else {
    *q_count = 0;
    counts[3] = 1;
  }
}

size_t check_tree_workspace_bytes(int n_nodes) {
  const size_t cap = (size_t)(n_nodes > 0 ? n_nodes : 1);
  return align_up(2 * cap * sizeof(int4), 256) + 256;
}

}  // namespace octgb

extern "C" {

OCT_API int oct_init_random_vec4_device(oct_vec4* d_points, int n, float min_coord, float range,
                                        int seed, oct_stream_t stream) {
  using namespace octgb;
  if (n < 0 || (n > 0 && (!d_points || (reinterpret_cast<uintptr_t>(d_points) & 15))))
    return OCT_ERR_INVALID_ARG;
  if (n == 0) return OCT_OK;
  int grid = (n + 255) / 256;
  if (grid > device_sm_count() * 16) grid = device_sm_count() * 16;
  init_random_vec4_kernel<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<float4*>(d_points), n, min_coord, range, (uint32_t)seed);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return OCT_ERR_CUDA;
  }
  return OCT_OK;
}

static int init_sequence(uint32_t* d_keys, int n, int descending, oct_stream_t stream) {
  using namespace octgb;
  if (n < 0 || (n > 0 && !d_keys)) return OCT_ERR_INVALID_ARG;
  if (n == 0) return OCT_OK;
  int grid = (n + 255) / 256;
  if (grid > device_sm_count() * 16) grid = device_sm_count() * 16;
  init_sequence_kernel<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(d_keys, n,
                                                                                descending);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return OCT_ERR_CUDA;
  }
  return OCT_OK;
}

OCT_API int oct_init_descending(uint32_t* d_keys, int n, oct_stream_t stream) {
  return init_sequence(d_keys, n, 1, stream);
}

OCT_API int oct_init_ascending(uint32_t* d_keys, int n, oct_stream_t stream) {
  return init_sequence(d_keys, n, 0, stream);
}

OCT_API int oct_morton_decode(const uint32_t* codes, int n, float min_coord, float range,
                              oct_vec4* d_out, oct_stream_t stream) {
  using namespace octgb;
  if (n < 0 || (n > 0 && (!codes || !d_out || (reinterpret_cast<uintptr_t>(d_out) & 15))))
    return OCT_ERR_INVALID_ARG;
  if (n == 0) return OCT_OK;
  int grid = (n + 255) / 256;
  if (grid > device_sm_count() * 16) grid = device_sm_count() * 16;
  morton_decode_kernel<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      codes, n, min_coord, range, reinterpret_cast<float4*>(d_out));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return OCT_ERR_CUDA;
  }
  return OCT_OK;
}

OCT_API size_t oct_check_tree_workspace_bytes(int n_nodes) {
  if (n_nodes < 0) return 0;
  return octgb::check_tree_workspace_bytes(n_nodes);
}

OCT_API int oct_check_tree(const oct_node* nodes, int n_nodes, const uint32_t* codes, int n_codes,
                           uint32_t root_prefix, int root_code_len, int root_index,
                           long long* d_counts, void* workspace, size_t workspace_bytes,
                           oct_stream_t stream) {
  using namespace octgb;
  if (n_nodes < 0 || n_codes < 0 || !d_counts || root_code_len < 0 || root_code_len > 30 ||
      (n_nodes > 0 && !nodes) || (n_codes > 0 && !codes) || !workspace ||
      (reinterpret_cast<uintptr_t>(workspace) & 255))
    return OCT_ERR_INVALID_ARG;
  if (workspace_bytes < check_tree_workspace_bytes(n_nodes)) return OCT_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const uint32_t cap = (uint32_t)(n_nodes > 0 ? n_nodes : 1);
  char* w = static_cast<char*>(workspace);
  uint32_t* qc = reinterpret_cast<uint32_t*>(w);  // [0] seed count, [1 + l] level l's output count
  int4* qa = reinterpret_cast<int4*>(w + 256);
  int4* qb = qa + cap;
  const int levels = (30 - root_code_len) / 3 + 1;
  unsigned long long* counts = reinterpret_cast<unsigned long long*>(d_counts);
  check_seed_kernel<<<1, 1, 0, s>>>(qa, qc, qc + 1, levels, root_index, root_prefix,
                                    root_code_len, n_nodes, counts);
  int grid = device_sm_count() * 8;
  const uint32_t* in_count = qc;
  int4* in = qa;
  int4* out = qb;
  for (int l = 0; l < levels; ++l) {
    check_level_kernel<<<grid, 256, 0, s>>>(nodes, n_nodes, codes, n_codes, in, in_count, out,
                                            qc + 1 + l, cap, counts);
    in_count = qc + 1 + l;
    int4* t = in;
    in = out;
    out = t;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return OCT_ERR_CUDA;
  }
  return OCT_OK;
}

}  // extern "C"
