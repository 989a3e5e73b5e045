// Host-side input generator: replaces k_InitRandomVec4 (reference
// include/kernels/00_init.hpp:10-11, kernels/00_init.cpp:20-30).
//
// The reference draws glm::vec4(dis(gen), dis(gen), dis(gen), 1) from
// std::mt19937(seed) and std::uniform_real_distribution<float>(min, min+range).
// The order in which the three draws land in x, y, z is whatever the compiler
// evaluates first; GCC evaluates the constructor arguments right to left, so
// the first draw is z. This file fixes that order explicitly so the points are
// the same on every compiler and host (the 1,048,576-point cloud of seed 114514
// starts (692.401062, 846.167542, 704.262024)). Compiled with
// -ffp-contract=off so the affine step is not fused on aarch64.
#include <random>

#include "octree_gb300.h"

extern "C" OCT_API void oct_init_random_vec4(oct_vec4* out, int n, float min_coord, float range,
                                             int seed) {
  if (!out || n <= 0) return;
  std::mt19937 gen(seed);
  std::uniform_real_distribution<float> dis(min_coord, min_coord + range);
  for (int i = 0; i < n; ++i) {
    const float z = dis(gen);
    const float y = dis(gen);
    const float x = dis(gen);
    out[i].x = x;
    out[i].y = y;
    out[i].z = z;
    out[i].w = 1.0f;
  }
}
