// ez_shim.h -- the few engine types that the reference's terrain noise code
// (source/math/Random.cpp, source/math/NoiseGenerator.cpp) uses, so that those
// files compile as they are, outside their engine.  TEST INFRASTRUCTURE: part
// of the oracle's pin to the reference, never linked into the product.
#pragma once
#include <stdint.h>

#include <algorithm>
#include <cmath>

typedef uint32_t ezUInt32;
typedef int32_t ezInt32;

struct ezVec3 {
  float x, y, z;
  ezVec3() = default;
  explicit ezVec3(float v) : x(v), y(v), z(v) {}
  ezVec3(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
  ezVec3 operator*(float s) const { return ezVec3(x * s, y * s, z * s); }
  ezVec3 operator+(const ezVec3& o) const { return ezVec3(x + o.x, y + o.y, z + o.z); }
};
inline ezVec3 operator*(float s, const ezVec3& v) { return v * s; }

#define EZ_ASSERT(cond, msg) ((void)0)
