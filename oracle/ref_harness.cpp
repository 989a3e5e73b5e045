// C-callable wrappers around the reference's own CPU stage functions.
//
// TEST INFRASTRUCTURE ONLY. This file is compiled together with the reference's
// unmodified kernels/*.cpp (by oracle/build_ref.sh, into oracle/_ref/) so that
// Python can call the reference implementation through ctypes. It is used to
// pin the C restatement in oracle/oracle.c and to generate the golden fixtures
// under tests/golden/. Nothing in the product links or loads it.
//
// Reference interfaces wrapped (paths within the reference project):
//   k_InitDescending      include/kernels/00_init.hpp:5, kernels/00_init.cpp:6-11
//   k_InitAscending       include/kernels/00_init.hpp:7, kernels/00_init.cpp:13-18
//   k_InitRandomVec4      include/kernels/00_init.hpp:10-11, kernels/00_init.cpp:20-30
//   k_ComputeMortonCode   include/kernels/01_morton.hpp:9-13
//   k_SimpleRadixSort     include/kernels/02_sort.hpp:6-7
//   k_SortKeysInplace     include/kernels/02_sort.hpp:5
//   k_CountUnique         include/kernels/03_unique.hpp:4
//   k_BuildRadixTree      include/kernels/04_radix_tree.hpp:5-11
//   k_EdgeCount           include/kernels/05_edge_count.hpp:5-8
//   k_PartialSum          include/kernels/06_partial_sum.hpp:6-9
//   k_MakeOctNodes        include/kernels/07_octree.hpp:5-14
//   k_LinkLeafNodes       include/kernels/07_octree.hpp:16-25
//   root-node set-up      apps/cpu_demo/main.cpp:125-132 (shared::morton32_to_xyz)
#include <omp.h>

#include <cstdint>
#include <cstring>

#include "kernels/all.hpp"
#include "shared/morton.h"
#include "shared/types.h"

static_assert(sizeof(OctNode) == 60, "OctNode is 60 bytes");

extern "C" {

void ref_set_threads(int n) { omp_set_num_threads(n); }

void ref_init_descending(unsigned* keys, int n) { k_InitDescending(keys, n); }

void ref_init_ascending(unsigned* keys, int n) { k_InitAscending(keys, n); }

void ref_init_random_vec4(float* out, int n, float min, float range, int seed) {
  k_InitRandomVec4(reinterpret_cast<glm::vec4*>(out), n, min, range, seed);
}

void ref_morton(const float* pts, unsigned* keys, long n, float min, float range) {
  k_ComputeMortonCode(reinterpret_cast<const glm::vec4*>(pts), keys, (size_t)n, min, range);
}

void ref_radix_sort(unsigned* keys, int n) { k_SimpleRadixSort(keys, n); }

void ref_radix_sort_alt(unsigned* keys, unsigned* alt, int n) { k_SimpleRadixSort(keys, alt, n); }

void ref_sort_inplace(unsigned* keys, int n) { k_SortKeysInplace(keys, n); }

int ref_count_unique(unsigned* keys, int n) { return k_CountUnique(keys, n); }

void ref_build_radix_tree(int n, const unsigned* codes, uint8_t* prefix_n, uint8_t* has_leaf_left,
                          uint8_t* has_leaf_right, int* left_child, int* parent) {
  k_BuildRadixTree(n, codes, prefix_n, reinterpret_cast<bool*>(has_leaf_left),
                   reinterpret_cast<bool*>(has_leaf_right), left_child, parent);
}

void ref_edge_count(const uint8_t* prefix_n, const int* parents, int* edge_count, int n) {
  k_EdgeCount(prefix_n, parents, edge_count, n);
}

void ref_partial_sum(const int* data, long first, long last, int* out) {
  (void)k_PartialSum(data, first, last, out);
}

// Root set-up exactly as apps/cpu_demo/main.cpp:125-132 does it.
void ref_root_init(void* nodes, const unsigned* sorted_codes, const uint8_t* prefix_n, float min,
                   float range) {
  OctNode* oct = static_cast<OctNode*>(nodes);
  const auto root_level = prefix_n[0] / 3;
  const auto root_prefix = sorted_codes[0] >> (morton_bits - (3 * root_level));
  shared::morton32_to_xyz(&oct[0].corner, root_prefix << (morton_bits - (3 * root_level)), min,
                          range);
  oct[0].cell_size = range;
}

void ref_make_oct_nodes(void* nodes, const int* offsets, const int* counts, const unsigned* codes,
                        const uint8_t* prefix_n, const int* parents, float min, float range,
                        int n) {
  k_MakeOctNodes(static_cast<OctNode*>(nodes), offsets, counts, codes, prefix_n, parents, min,
                 range, n);
}

void ref_link_leaf_nodes(void* nodes, const int* offsets, const int* counts, const unsigned* codes,
                         const uint8_t* has_leaf_left, const uint8_t* has_leaf_right,
                         const uint8_t* prefix_n, const int* parents, const int* left_child,
                         int n) {
  k_LinkLeafNodes(static_cast<OctNode*>(nodes), offsets, counts, codes,
                  reinterpret_cast<const bool*>(has_leaf_left),
                  reinterpret_cast<const bool*>(has_leaf_right), prefix_n, parents, left_child, n);
}

}  // extern "C"
