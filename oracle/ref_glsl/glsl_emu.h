// glsl_emu.h -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// A minimal GLSL 4.30 compute-shader environment written as C++, so that the
// reference's own shader files (terrainwatersim/shader/flowUpdate.comp,
// flowApply.comp, waterBrush.comp, simulationCommon.glsl) compile unchanged as
// C++ and run on the CPU.  oracle/Makefile feeds each shader to g++ with this
// header force-included and the `#version` line dropped; the resulting
// library (oracle/_ref/libtws_ref.so) is the reference itself, run here, and is
// used to pin the oracle restatement and to make tests/golden fixtures.
//
// Semantics emulated (OpenGL 4.3 core, GLSL 4.30):
//   * image2D rgba32f / rg16f with imageLoad/imageStore; an out-of-range load
//     returns zero and an out-of-range store has no effect (GL 4.3 section 8.26).
//     rg16f stores round to the nearest half (ties to even).
//   * One dispatch runs its workgroups one after another.  Inside a workgroup,
//     barrier() is emulated in two passes: pass 0 runs every invocation up to
//     its barrier() (filling `shared` arrays), pass 1 runs every invocation
//     again with barrier() a no-op.  This is exact for these shaders because
//     everything before their barrier() is a pure load of data the dispatch does
//     not write, so re-running it stores the same values.
//   * max(x, y) = (x < y) ? y : x, clamp(x, lo, hi) = min(max(x, lo), hi),
//     dot(a, b) = a.x*b.x + a.y*b.y, vec/ivec operators per component.
// Build with -ffp-contract=off so that no multiply-add is fused.

#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

typedef unsigned int uint;

struct vec2;
struct ivec2;

struct bvec2 {
  bool x, y;
};

struct uvec2 {
  uint x, y;
  uvec2() : x(0), y(0) {}
  explicit uvec2(uint s) : x(s), y(s) {}
  uvec2(uint a, uint b) : x(a), y(b) {}
};

// gl_WorkGroupID and friends: x, y, z plus the .xy swizzle the shaders read
// (kept consistent by the dispatcher).
struct glsl_uvec3 {
  uint x, y, z;
  uvec2 xy;
  void set(uint a, uint b, uint c) {
    x = a;
    y = b;
    z = c;
    xy = uvec2(a, b);
  }
};

struct ivec2 {
  int x, y;
  ivec2() : x(0), y(0) {}
  explicit ivec2(int s) : x(s), y(s) {}
  ivec2(int a, int b) : x(a), y(b) {}
  explicit ivec2(const uvec2& u) : x((int)u.x), y((int)u.y) {}
};
inline ivec2 operator+(ivec2 a, ivec2 b) { return ivec2(a.x + b.x, a.y + b.y); }
inline ivec2 operator-(ivec2 a, ivec2 b) { return ivec2(a.x - b.x, a.y - b.y); }
inline ivec2 operator*(ivec2 a, ivec2 b) { return ivec2(a.x * b.x, a.y * b.y); }

struct vec2 {
  float x, y;
  vec2() : x(0), y(0) {}
  explicit vec2(float s) : x(s), y(s) {}
  vec2(float a, float b) : x(a), y(b) {}
};
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
// GLSL converts the ivec2 operand to vec2 implicitly (waterBrush.comp:26).
inline vec2 operator-(vec2 a, ivec2 b) { return vec2(a.x - (float)b.x, a.y - (float)b.y); }
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }

template <int A, int B>
struct glsl_swz2 {
  float v[4];
  glsl_swz2& operator=(const vec2& o) {
    v[A] = o.x;
    v[B] = o.y;
    return *this;
  }
  // swizzle = swizzle writes only the two named components
  glsl_swz2& operator=(const glsl_swz2& o) { return *this = vec2(o.v[A], o.v[B]); }
  operator vec2() const { return vec2(v[A], v[B]); }
};

inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator*(float s, vec2 a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator+(float s, vec2 a) { return vec2(s + a.x, s + a.y); }

// vec3 with the .xz / .xy swizzles the water shaders assign through.
struct vec3 {
  union {
    struct {
      float x, y, z;
    };
    glsl_swz2<0, 2> xz;
    glsl_swz2<0, 1> xy;
  };
  vec3() { x = y = z = 0.0f; }
  vec3(float a0, float a1, float a2) {
    x = a0;
    y = a1;
    z = a2;
  }
  vec3(const vec3& o) { std::memcpy(this, &o, sizeof(vec3)); }
  vec3& operator=(const vec3& o) {
    std::memcpy(this, &o, sizeof(vec3));
    return *this;
  }
};
inline vec3 operator/(const vec3& v, float s) { return vec3(v.x / s, v.y / s, v.z / s); }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// GLSL 4.30 section 8.5: cross(x, y) = (x1 y2 - y1 x2, x2 y0 - y2 x0, x0 y1 - y0 x1)
inline vec3 cross(const vec3& a, const vec3& b) {
  return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float sqrt(float v) { return std::sqrt(v); }
// normalize and length are implementation-defined in precision (GLSL 4.30
// section 4.7.1); this emulation takes v / sqrt(dot(v, v)), correctly rounded
// at each operation.
inline vec3 normalize(const vec3& v) { return v / sqrt(dot(v, v)); }

struct vec4 {
  union {
    struct {
      float x, y, z, w;
    };
    struct {
      float r, g, b, a;
    };
    glsl_swz2<2, 3> zw;
    glsl_swz2<0, 1> xy;
  };
  vec4() { x = y = z = w = 0.0f; }
  vec4(const vec3& v, float a3) {
    x = v.x;
    y = v.y;
    z = v.z;
    w = a3;
  }
  explicit vec4(float s) { x = y = z = w = s; }
  vec4(float a0, float a1, float a2, float a3) {
    x = a0;
    y = a1;
    z = a2;
    w = a3;
  }
  vec4(const vec4& o) { std::memcpy(this, &o, sizeof(vec4)); }
  vec4& operator=(const vec4& o) {
    std::memcpy(this, &o, sizeof(vec4));
    return *this;
  }
  float& operator[](int i) { return (&x)[i]; }
  float operator[](int i) const { return (&x)[i]; }
  vec4& operator*=(float s) {
    x = x * s;
    y = y * s;
    z = z * s;
    w = w * s;
    return *this;
  }
};
inline vec4 operator*(const vec4& v, float s) { return vec4(v.x * s, v.y * s, v.z * s, v.w * s); }
inline vec4 operator+(const vec4& a, const vec4& b) {
  return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

inline float glsl_maxf(float x, float y) { return (x < y) ? y : x; }
inline float glsl_minf(float x, float y) { return (y < x) ? y : x; }
inline vec4 max(const vec4& p, const vec4& q) {
  return vec4(glsl_maxf(p.x, q.x), glsl_maxf(p.y, q.y), glsl_maxf(p.z, q.z), glsl_maxf(p.w, q.w));
}
inline float max(int x, float y) { return glsl_maxf((float)x, y); }
inline float max(float x, float y) { return glsl_maxf(x, y); }
inline float clamp(float v, int lo, int hi) { return glsl_minf(glsl_maxf(v, (float)lo), (float)hi); }
inline bvec2 equal(uvec2 a, uvec2 b) { return bvec2{a.x == b.x, a.y == b.y}; }
inline bool any(bvec2 v) { return v.x || v.y; }

// IEEE binary16 from float, round to nearest, ties to even (written out so the
// result does not depend on the host's half-precision support).
inline uint16_t glsl_float_to_half(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  const uint32_t sign = (u >> 16) & 0x8000u;
  const uint32_t ax = u & 0x7fffffffu;
  if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // rounds to >= 65520 -> inf
  if (ax < 0x38800000u) {                                     // half subnormal or zero
    if (ax < 0x33000000u) return (uint16_t)sign;              // < 2^-25 -> 0
    const uint32_t e = ax >> 23;
    const uint32_t m = (ax & 0x7fffffu) | 0x800000u;
    const uint32_t shift = 126u - e;  // value = m * 2^(e-150) = (m >> shift) * 2^-24
    uint32_t h = m >> shift;
    const uint32_t rem = m & ((1u << shift) - 1u);
    const uint32_t halfway = 1u << (shift - 1u);
    if (rem > halfway || (rem == halfway && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
  }
  uint32_t h = ((ax - 0x38000000u) >> 13);  // rebias exponent 127 -> 15
  const uint32_t rem = ax & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
  return (uint16_t)(sign | h);
}

enum glsl_format { GLSL_RGBA32F = 0, GLSL_RG16F = 1 };

struct image2D {
  void* data = nullptr;
  int width = 0, height = 0;
  int format = GLSL_RGBA32F;
};

inline vec4 imageLoad(const image2D& img, ivec2 p) {
  if (p.x < 0 || p.y < 0 || p.x >= img.width || p.y >= img.height) return vec4(0.0f);
  const float* t = static_cast<const float*>(img.data) + 4 * ((size_t)p.y * img.width + p.x);
  return vec4(t[0], t[1], t[2], t[3]);
}

inline void imageStore(image2D& img, ivec2 p, const vec4& v) {
  if (p.x < 0 || p.y < 0 || p.x >= img.width || p.y >= img.height) return;
  const size_t i = (size_t)p.y * img.width + p.x;
  if (img.format == GLSL_RGBA32F) {
    float* t = static_cast<float*>(img.data) + 4 * i;
    t[0] = v.x;
    t[1] = v.y;
    t[2] = v.z;
    t[3] = v.w;
  } else {
    uint16_t* t = static_cast<uint16_t*>(img.data) + 2 * i;
    t[0] = glsl_float_to_half(v.x);
    t[1] = glsl_float_to_half(v.y);
  }
}

// Invocation state set by the dispatcher.
static glsl_uvec3 gl_WorkGroupID, gl_LocalInvocationID, gl_GlobalInvocationID;
static int glsl_emu_pass = 1;

// GLSL qualifiers that have no C++ meaning here.
#define layout(...)
#define restrict
#define readonly
#define writeonly
#define uniform
#define in
#define shared static
// Uniform blocks become namespace-scope variables: `Name { members };` turns
// into `namespace { members };`.
#define SimulationParameters namespace
#define BrushInfo namespace
// Two-pass workgroup barrier (see the header comment).
#define barrier()          \
  do {                     \
    if (glsl_emu_pass == 0) \
      return;              \
  } while (0)
