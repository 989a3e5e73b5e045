// octree_gb300_kernels.hpp — drop-in for the reference's per-stage entry
// points (ucsc-redwood/pipeline include/kernels/all.hpp), header-only, over
// the C ABI of libpipeline_gb300.so (octree_gb300.h).
//
// A caller written against the reference, e.g. apps/cpu_demo/main.cpp:72-154,
// includes this header instead of "kernels/all.hpp" and links
// libpipeline_gb300.so plus the CUDA runtime; the calls keep their names,
// argument order and meaning. glm::vec4 and OctNode are taken as template
// parameters (any 16-byte float4 / 60-byte OctNode layout is accepted), so no
// glm dependency is added.
//
// Memory: the reference's CPU functions take host pointers and its GPU driver
// passes managed memory (apps/gpu_demo/main.cu:13-23). Here each call accepts
// either: device or managed pointers are used in place; plain host pointers
// are copied to temporary device buffers and back. Every call is synchronous
// on the legacy stream, as the reference's functions return with the work
// done. Errors throw std::runtime_error (the reference has no error path).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "octree_gb300.h"

namespace octree_gb300_detail {

inline void cuda_ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

inline void oct_ok(int rc, const char* what) {
  if (rc != OCT_OK) {
    std::string m = std::string(what) + ": oct_status " + std::to_string(rc);
    if (rc == OCT_ERR_CUDA) m += std::string(" (") + oct_last_error() + ")";
    throw std::runtime_error(m);
  }
}

inline bool on_device(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// A device view of a caller buffer: the buffer itself, or a temporary copy.
template <class T>
class DeviceView {
  using U = std::remove_const_t<T>;

 public:
  DeviceView(T* user, size_t count, bool copy_in) : user_(const_cast<U*>(user)), count_(count) {
    if (count == 0 || on_device(user)) {
      dev_ = user_;
      return;
    }
    cuda_ok(cudaMalloc(reinterpret_cast<void**>(&dev_), sizeof(T) * count), "cudaMalloc");
    owned_ = true;
    if (copy_in)
      cuda_ok(cudaMemcpy(dev_, user_, sizeof(T) * count, cudaMemcpyHostToDevice), "copy in");
  }
  ~DeviceView() {
    if (owned_) cudaFree(dev_);
  }
  DeviceView(const DeviceView&) = delete;
  DeviceView& operator=(const DeviceView&) = delete;
  T* get() const { return dev_; }
  void copy_out() {
    cuda_ok(cudaDeviceSynchronize(), "synchronize");
    if (owned_)
      cuda_ok(cudaMemcpy(user_, dev_, sizeof(T) * count_, cudaMemcpyDeviceToHost), "copy out");
  }

 private:
  U* user_;
  U* dev_ = nullptr;
  size_t count_;
  bool owned_ = false;
};

inline void* workspace(size_t bytes, std::vector<void*>& keep) {
  void* p = nullptr;
  if (bytes) cuda_ok(cudaMalloc(&p, bytes), "cudaMalloc workspace");
  keep.push_back(p);
  return p;
}

struct Frees {
  std::vector<void*> ptrs;
  ~Frees() {
    for (void* p : ptrs) cudaFree(p);
  }
};

// One past the largest OctNode slot stages 7-8 write (contract O3), from
// host-visible or device edge counts / prefix sums.
inline int oct_node_count(const int* counts, const int* offsets, int n) {
  if (n <= 0) return 0;
  DeviceView<const int> ec(counts, n, true), ps(offsets, n, true);
  int* d = nullptr;
  cuda_ok(cudaMalloc(reinterpret_cast<void**>(&d), sizeof(int)), "cudaMalloc");
  int h = 0;
  const int rc = oct_octree_node_count(ec.get(), ps.get(), n, d, nullptr);
  cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  oct_ok(rc, "node count");
  return h;
}

}  // namespace octree_gb300_detail

// include/kernels/00_init.hpp:5 (keys[i] = n - i).
inline void k_InitDescending(unsigned int* sort, int n) {
  namespace d = octree_gb300_detail;
  d::DeviceView<unsigned int> out(sort, n > 0 ? (size_t)n : 0, false);
  d::oct_ok(oct_init_descending(out.get(), n, nullptr), "k_InitDescending");
  out.copy_out();
}

// include/kernels/00_init.hpp:7 (keys[i] = i).
inline void k_InitAscending(unsigned int* sort, int n) {
  namespace d = octree_gb300_detail;
  d::DeviceView<unsigned int> out(sort, n > 0 ? (size_t)n : 0, false);
  d::oct_ok(oct_init_ascending(out.get(), n, nullptr), "k_InitAscending");
  out.copy_out();
}

// include/kernels/00_init.hpp:10-11 (host generator).
template <class Vec4>
inline void k_InitRandomVec4(Vec4* u_data, int n, float min, float range, int seed) {
  static_assert(sizeof(Vec4) == 16, "expects glm::vec4 (four floats)");
  namespace d = octree_gb300_detail;
  if (d::on_device(u_data)) {
    std::vector<oct_vec4> tmp(n > 0 ? n : 0);
    oct_init_random_vec4(tmp.data(), n, min, range, seed);
    d::cuda_ok(cudaMemcpy(u_data, tmp.data(), sizeof(oct_vec4) * tmp.size(), cudaMemcpyHostToDevice),
               "copy");
  } else {
    oct_init_random_vec4(reinterpret_cast<oct_vec4*>(u_data), n, min, range, seed);
  }
}

// include/kernels/01_morton.hpp:9-13.
template <class Vec4>
inline void k_ComputeMortonCode(const Vec4* data, unsigned int* morton_keys, size_t n,
                                float min_coord, float range) {
  static_assert(sizeof(Vec4) == 16, "expects glm::vec4 (four floats)");
  namespace d = octree_gb300_detail;
  d::DeviceView<const Vec4> in(data, n, true);
  d::DeviceView<unsigned int> out(morton_keys, n, false);
  d::oct_ok(oct_morton_encode(reinterpret_cast<const oct_vec4*>(in.get()), out.get(), (int64_t)n,
                              min_coord, range, nullptr, nullptr),
            "k_ComputeMortonCode");
  out.copy_out();
}

// include/kernels/02_sort.hpp:5-7.
inline void k_SimpleRadixSort(unsigned int* keys, unsigned int* keys_alt, int n) {
  namespace d = octree_gb300_detail;
  d::Frees f;
  d::DeviceView<unsigned int> k(keys, n, true);
  unsigned int* alt = keys_alt && d::on_device(keys_alt)
                          ? keys_alt
                          : static_cast<unsigned int*>(d::workspace(sizeof(unsigned) * n, f.ptrs));
  const size_t wb = oct_sort_workspace_bytes(n, 32);
  void* ws = d::workspace(wb, f.ptrs);
  d::oct_ok(oct_sort_keys(k.get(), alt, n, 32, ws, wb, nullptr, nullptr), "k_SimpleRadixSort");
  k.copy_out();
}
inline void k_SimpleRadixSort(unsigned int* keys, int n) { k_SimpleRadixSort(keys, nullptr, n); }
inline void k_SortKeysInplace(unsigned int* keys, int n) { k_SimpleRadixSort(keys, nullptr, n); }

// include/kernels/03_unique.hpp:4.
[[nodiscard]] inline int k_CountUnique(unsigned int* keys, int n) {
  namespace d = octree_gb300_detail;
  d::Frees f;
  d::DeviceView<unsigned int> k(keys, n, true);
  int* du = static_cast<int*>(d::workspace(sizeof(int), f.ptrs));
  const size_t wb = oct_unique_workspace_bytes(n);
  void* ws = d::workspace(wb, f.ptrs);
  d::oct_ok(oct_unique(k.get(), n, du, ws, wb, nullptr, nullptr), "k_CountUnique");
  k.copy_out();
  int u = 0;
  d::cuda_ok(cudaMemcpy(&u, du, sizeof(int), cudaMemcpyDeviceToHost), "copy");
  return u;
}

// include/kernels/04_radix_tree.hpp:5-11 (n = number of radix nodes = U - 1).
inline void k_BuildRadixTree(int n, const unsigned int* codes, uint8_t* prefix_n,
                             bool* has_leaf_left, bool* has_leaf_right, int* left_child,
                             int* parent) {
  namespace d = octree_gb300_detail;
  d::DeviceView<const unsigned int> c(codes, (size_t)n + 1, true);
  d::DeviceView<uint8_t> pn(prefix_n, n, false);
  d::DeviceView<bool> hl(has_leaf_left, n, false), hr(has_leaf_right, n, false);
  d::DeviceView<int> lc(left_child, n, false), pa(parent, n, false);
  d::oct_ok(oct_build_radix_tree(n, c.get(), pn.get(), reinterpret_cast<uint8_t*>(hl.get()),
                                 reinterpret_cast<uint8_t*>(hr.get()), lc.get(), pa.get(), nullptr),
            "k_BuildRadixTree");
  pn.copy_out();
  hl.copy_out();
  hr.copy_out();
  lc.copy_out();
  pa.copy_out();
}

// include/kernels/05_edge_count.hpp:5-8.
inline void k_EdgeCount(const uint8_t* prefix_n, const int* parents, int* edge_count,
                        int n_brt_nodes) {
  namespace d = octree_gb300_detail;
  d::DeviceView<const uint8_t> pn(prefix_n, n_brt_nodes, true);
  d::DeviceView<const int> pa(parents, n_brt_nodes, true);
  d::DeviceView<int> ec(edge_count, n_brt_nodes, false);
  d::oct_ok(oct_edge_count(pn.get(), pa.get(), ec.get(), n_brt_nodes, nullptr), "k_EdgeCount");
  ec.copy_out();
}

// include/kernels/06_partial_sum.hpp:6-9: returns one past the last output.
[[nodiscard]] inline int* k_PartialSum(const int* data, std::ptrdiff_t first, std::ptrdiff_t last,
                                       int* d_first) {
  namespace d = octree_gb300_detail;
  const int n = (int)(last - first);
  if (n <= 0) return d_first;
  d::Frees f;
  d::DeviceView<const int> in(data + first, n, true);
  d::DeviceView<int> out(d_first, n, false);
  const size_t wb = oct_prefix_sum_workspace_bytes(n);
  void* ws = d::workspace(wb, f.ptrs);
  d::oct_ok(oct_prefix_sum(in.get(), n, out.get(), ws, wb, nullptr, nullptr), "k_PartialSum");
  out.copy_out();
  return d_first + n;
}

// include/kernels/07_octree.hpp:5-14 (N = number of radix nodes). The node
// array holds the OctNodes the tree needs (contract O3), initialised by the
// caller as apps/cpu_demo/main.cpp:123-132 does.
template <class Node>
inline void k_MakeOctNodes(Node* oct_nodes, const int* node_offsets, const int* rt_node_counts,
                           const unsigned int* codes, const uint8_t* rt_prefixN,
                           const int* rt_parents, float min_coord, float range, int N) {
  static_assert(sizeof(Node) == sizeof(oct_node), "expects OctNode (60 bytes)");
  namespace d = octree_gb300_detail;
  const int m = d::oct_node_count(rt_node_counts, node_offsets, N);
  d::Frees f;
  d::DeviceView<Node> nodes(oct_nodes, m, true);
  d::DeviceView<const int> ps(node_offsets, N, true), ec(rt_node_counts, N, true),
      pa(rt_parents, N, true);
  d::DeviceView<const unsigned int> c(codes, (size_t)N + 1, true);
  d::DeviceView<const uint8_t> pn(rt_prefixN, N, true);
  const size_t wb = oct_octree_workspace_bytes(m);
  void* ws = d::workspace(wb, f.ptrs);
  d::oct_ok(oct_make_oct_nodes(reinterpret_cast<oct_node*>(nodes.get()), m, ps.get(), ec.get(),
                               c.get(), pn.get(), pa.get(), min_coord, range, N, ws, wb, nullptr,
                               nullptr),
            "k_MakeOctNodes");
  nodes.copy_out();
}

// include/kernels/07_octree.hpp:16-25.
template <class Node>
inline void k_LinkLeafNodes(Node* nodes, const int* node_offsets, const int* rt_node_counts,
                            const unsigned int* codes, const bool* rt_hasLeafLeft,
                            const bool* rt_hasLeafRight, const uint8_t* rt_prefixN,
                            const int* rt_parents, const int* rt_leftChild, int N) {
  static_assert(sizeof(Node) == sizeof(oct_node), "expects OctNode (60 bytes)");
  namespace d = octree_gb300_detail;
  const int m = d::oct_node_count(rt_node_counts, node_offsets, N);
  d::Frees f;
  d::DeviceView<Node> nd(nodes, m, true);
  d::DeviceView<const int> ps(node_offsets, N, true), ec(rt_node_counts, N, true),
      pa(rt_parents, N, true), lc(rt_leftChild, N, true);
  d::DeviceView<const unsigned int> c(codes, (size_t)N + 1, true);
  d::DeviceView<const bool> hl(rt_hasLeafLeft, N, true), hr(rt_hasLeafRight, N, true);
  d::DeviceView<const uint8_t> pn(rt_prefixN, N, true);
  const size_t wb = oct_octree_workspace_bytes(m);
  void* ws = d::workspace(wb, f.ptrs);
  d::oct_ok(oct_link_leaf_nodes(reinterpret_cast<oct_node*>(nd.get()), m, ps.get(), ec.get(),
                                c.get(), reinterpret_cast<const uint8_t*>(hl.get()),
                                reinterpret_cast<const uint8_t*>(hr.get()), pn.get(), pa.get(),
                                lc.get(), N, ws, wb, nullptr, nullptr),
            "k_LinkLeafNodes");
  nd.copy_out();
}
