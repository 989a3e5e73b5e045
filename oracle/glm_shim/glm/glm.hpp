// Minimal stand-in for <glm/glm.hpp>, written for this project so that the
// reference's CPU stage sources compile without the glm package.
//
// The reference uses glm only as storage: `glm::vec4` (four floats, 16 bytes,
// indexable with operator[] and constructible from four floats). Nothing else
// of glm is touched by include/shared/{morton,oct,types}.h or kernels/*.cpp.
#pragma once

#include <cstddef>
#include <cstdint>

namespace glm {

struct vec4 {
  float x, y, z, w;

  vec4() = default;
  constexpr vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}

  float& operator[](std::size_t i) { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
  const float& operator[](std::size_t i) const {
    return i == 0 ? x : i == 1 ? y : i == 2 ? z : w;
  }
};

static_assert(sizeof(vec4) == 16, "glm::vec4 is four packed floats");

}  // namespace glm
