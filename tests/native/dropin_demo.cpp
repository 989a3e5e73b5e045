// The reference's CPU demo call sequence (apps/cpu_demo/main.cpp:63-154),
// written against octree_gb300_kernels.hpp instead of "kernels/all.hpp":
// same function names, argument order and host buffers. Prints the sizes and
// an FNV-1a-64 hash of every stage buffer so a test can compare them with the
// golden values of the reference itself.
//
// Build: g++ -std=c++17 -O2 -I include -I <cuda>/include dropin_demo.cpp
//        -L pipeline_gb300/_lib -lpipeline_gb300 -L <cuda>/lib64 -lcudart
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "octree_gb300_kernels.hpp"

namespace glm {
struct vec4 {
  float x, y, z, w;
};
}  // namespace glm

struct OctNode {
  int children[8];
  glm::vec4 corner;
  float cell_size;
  int child_node_mask;
  int child_leaf_mask;
};

static uint64_t fnv(const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

int main(int argc, char** argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : (1 << 20);
  constexpr float min = 0.0f, range = 1024.0f;
  std::vector<glm::vec4> u_input(n);
  std::vector<unsigned int> u_sort(n);
  k_InitRandomVec4(u_input.data(), n, min, range, 114514);
  k_ComputeMortonCode(u_input.data(), u_sort.data(), n, min, range);
  std::printf("morton %016llx\n", (unsigned long long)fnv(u_sort.data(), 4ull * n));
  k_SimpleRadixSort(u_sort.data(), n);
  const int n_unique = k_CountUnique(u_sort.data(), n);
  const int B = n_unique - 1;
  std::vector<uint8_t> prefix(B);
  std::vector<uint8_t> hll_b(B), hlr_b(B);
  bool* hll = reinterpret_cast<bool*>(hll_b.data());
  bool* hlr = reinterpret_cast<bool*>(hlr_b.data());
  std::vector<int> left(B), parent(B, 0), ec(B), ps(B);
  k_BuildRadixTree(B, u_sort.data(), prefix.data(), hll, hlr, left.data(), parent.data());
  k_EdgeCount(prefix.data(), parent.data(), ec.data(), B);
  (void)k_PartialSum(ec.data(), 0, B, ps.data());
  ps[0] = 0;
  int m = ps[B - 1];
  for (int i = 1; i < B; ++i)
    if (ec[i] > 0 && ps[i] + ec[i] - 1 > m) m = ps[i] + ec[i] - 1;
  m += 1;
  std::vector<OctNode> nodes(m);
  std::memset(nodes.data(), 0, sizeof(OctNode) * m);
  // root set-up (apps/cpu_demo/main.cpp:125-132) through the device helper
  {
    OctNode* d_nodes = nullptr;
    unsigned* d_codes = nullptr;
    uint8_t* d_prefix = nullptr;
    cudaMalloc(&d_nodes, sizeof(OctNode) * m);
    cudaMalloc(&d_codes, 4);
    cudaMalloc(&d_prefix, 1);
    cudaMemcpy(d_nodes, nodes.data(), sizeof(OctNode) * m, cudaMemcpyHostToDevice);
    cudaMemcpy(d_codes, u_sort.data(), 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_prefix, prefix.data(), 1, cudaMemcpyHostToDevice);
    oct_octree_root_init(reinterpret_cast<oct_node*>(d_nodes), d_codes, d_prefix, min, range,
                         nullptr);
    k_MakeOctNodes(d_nodes, ps.data(), ec.data(), u_sort.data(), prefix.data(), parent.data(), min,
                   range, B);
    k_LinkLeafNodes(d_nodes, ps.data(), ec.data(), u_sort.data(), hll, hlr, prefix.data(),
                    parent.data(), left.data(), B);
    cudaMemcpy(nodes.data(), d_nodes, sizeof(OctNode) * m, cudaMemcpyDeviceToHost);
    cudaFree(d_nodes);
    cudaFree(d_codes);
    cudaFree(d_prefix);
  }
  std::printf("n_unique %d\nn_oct %d\n", n_unique, m);
  std::printf("sorted_unique %016llx\n", (unsigned long long)fnv(u_sort.data(), 4ull * n_unique));
  std::printf("keys_after_unique %016llx\n", (unsigned long long)fnv(u_sort.data(), 4ull * n));
  std::printf("prefix_n %016llx\n", (unsigned long long)fnv(prefix.data(), B));
  std::printf("has_leaf_left %016llx\n", (unsigned long long)fnv(hll_b.data(), B));
  std::printf("has_leaf_right %016llx\n", (unsigned long long)fnv(hlr_b.data(), B));
  std::printf("left_child %016llx\n", (unsigned long long)fnv(left.data(), 4ull * B));
  std::printf("parent %016llx\n", (unsigned long long)fnv(parent.data(), 4ull * B));
  std::printf("edge_count %016llx\n", (unsigned long long)fnv(ec.data(), 4ull * B));
  std::printf("prefix_sum %016llx\n", (unsigned long long)fnv(ps.data(), 4ull * B));
  std::printf("oct_nodes %016llx\n", (unsigned long long)fnv(nodes.data(), sizeof(OctNode) * m));
  return 0;
}
