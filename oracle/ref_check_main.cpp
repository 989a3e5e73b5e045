// Driver that runs the reference's own checkTree (apps/cpu_demo/main.cpp:13-35)
// on an octree read from a file.
//
// TEST INFRASTRUCTURE ONLY. oracle/build_ref.sh compiles it together with the
// reference's unmodified apps/cpu_demo/main.cpp (its main renamed by
// -Dmain=ref_demo_main, its CLI11 and spdlog includes served by the stand-ins
// in oracle/ref_check/) and kernels/*.cpp into oracle/_ref/ref_check.
// tests/golden/make_check_tree.py counts the "oh no..." lines checkTree prints
// (one per leaf whose code does not carry its octant's prefix) to make the
// fixtures in tests/golden/check_tree.json.
//
// Input file (little-endian): int32 n_nodes, n_nodes x 60-byte OctNode,
// int32 n_codes, n_codes x uint32 codes, uint32 prefix, int32 code_len,
// int32 root. The caller guarantees that every step checkTree takes stays
// inside the arrays and within 30 code bits (the oracle's own check reports
// no rejected step for the input), so the recursion ends.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "shared/types.h"

void checkTree(const unsigned int prefix, const int code_len, const OctNode* nodes,
               const int oct_idx, const unsigned int* codes);

static_assert(sizeof(OctNode) == 60, "OctNode is 60 bytes");

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: ref_check FILE\n");
    return 2;
  }
  std::FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int32_t n_nodes = 0, n_codes = 0, code_len = 0, root = 0;
  uint32_t prefix = 0;
  bool ok = std::fread(&n_nodes, 4, 1, f) == 1 && n_nodes > 0;
  std::vector<OctNode> nodes(ok ? n_nodes : 0);
  ok = ok && std::fread(nodes.data(), sizeof(OctNode), nodes.size(), f) == nodes.size();
  ok = ok && std::fread(&n_codes, 4, 1, f) == 1 && n_codes > 0;
  std::vector<unsigned int> codes(ok ? n_codes : 0);
  ok = ok && std::fread(codes.data(), 4, codes.size(), f) == codes.size();
  ok = ok && std::fread(&prefix, 4, 1, f) == 1 && std::fread(&code_len, 4, 1, f) == 1 &&
       std::fread(&root, 4, 1, f) == 1;
  std::fclose(f);
  if (!ok || root < 0 || root >= n_nodes) return 2;
  checkTree(prefix, code_len, nodes.data(), root, codes.data());
  std::fflush(stdout);
  return 0;
}
