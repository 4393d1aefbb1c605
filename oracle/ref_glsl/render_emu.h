// render_emu.h -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// What the reference's water-rendering shaders need, beyond glsl_emu.h, for
// the parts of them that read the simulation's textures to compile as C++ and
// run on the CPU (oracle/Makefile, target `ref`):
//   waterRender.vert   the whole file (its patch placement comes from the
//                      stand-in ref_glsl/landscapeRenderFunctions.glsl)
//   waterRender.eval   its main() (the tessellation interface it reads and
//                      writes is declared in dispatch_waterRender_eval.inc)
//   waterRender.frag   ComputeHeightmapNormal and the flow-speed lines of
//                      main() (the rest of the fragment shader is lighting)
// Force-included after glsl_emu.h.  The shaders' float literals are single
// precision as in GLSL: the Makefile compiles these files with
// -fsingle-precision-constant.
//
// Texture sampling: the tests sample at texel centres only (coordinates
// (i + 0.5) / size, exact for power-of-two sizes), where a linear filter
// returns the texel itself; texture() and textureLod() return the texel whose
// centre the coordinate names, wrapping under the REPEAT mode the renderer
// binds for these textures (Terrain.cpp:112-113, 313-317).  A coordinate
// that is not a texel centre returns NaN, so a test that strays from centres
// fails instead of silently disagreeing with a GL filter.
#pragma once

#include <cmath>

struct mat4 {
  vec4 c[4];  // columns
};
inline vec4 operator*(const mat4& m, const vec4& v) {
  return vec4(m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z + m.c[3].x * v.w,
              m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z + m.c[3].y * v.w,
              m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z + m.c[3].z * v.w,
              m.c[0].w * v.x + m.c[1].w * v.y + m.c[2].w * v.z + m.c[3].w * v.w);
}

enum glsl_tex_format { GLSL_TEX_RGBA32F = 0, GLSL_TEX_RG16F = 1 };

struct sampler2D {
  const void* data = nullptr;
  int width = 0, height = 0;
  int format = GLSL_TEX_RGBA32F;
};

inline float glsl_half_to_float(uint16_t h) {
  const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  const uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
  float f;
  if (e == 0) {
    f = std::ldexp((float)m, -24);  // zero or subnormal, exact
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u |= sign;
    std::memcpy(&f, &u, 4);
    return f;
  }
  uint32_t u = e == 31 ? (sign | 0x7f800000u | (m << 13)) : (sign | ((e + 112u) << 23) | (m << 13));
  std::memcpy(&f, &u, 4);
  return f;
}

inline int glsl_texel_index(float coord, int size, bool* ok) {
  const float t = coord * (float)size - 0.5f;
  const float r = std::floor(t + 0.5f);
  if (std::fabs(t - r) > 1e-3f) *ok = false;
  int i = (int)r % size;
  return i < 0 ? i + size : i;
}

inline vec4 texture(const sampler2D& s, vec2 uv) {
  bool ok = true;
  const int i = glsl_texel_index(uv.x, s.width, &ok), j = glsl_texel_index(uv.y, s.height, &ok);
  if (!ok || !s.data) return vec4(NAN);
  const size_t k = (size_t)j * s.width + i;
  if (s.format == GLSL_TEX_RG16F) {
    const uint16_t* t = static_cast<const uint16_t*>(s.data) + 2 * k;
    return vec4(glsl_half_to_float(t[0]), glsl_half_to_float(t[1]), 0.0f, 1.0f);
  }
  const float* t = static_cast<const float*>(s.data) + 4 * k;
  return vec4(t[0], t[1], t[2], t[3]);
}
// Level 0 is the texture itself; the calls read level 0 only.
inline vec4 textureLod(const sampler2D& s, vec2 uv, float lod) {
  return lod == 0.0f ? texture(s, uv) : vec4(NAN);
}

// GLSL qualifiers of the render stages.
#define out
// Uniform blocks become namespace-scope variables (see glsl_emu.h).
#define GlobalLandscapeInfo namespace
