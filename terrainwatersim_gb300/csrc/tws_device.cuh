// tws_device.cuh -- device arithmetic shared by every libtws kernel.
//
// All floating-point operations of the simulation go through these helpers:
// IEEE round-to-nearest with no multiply-add contraction, so every kernel is
// bit-identical to the FP32 CPU transcription of the reference shaders.
#pragma once
#include "tws_internal.h"

namespace tws {

// ---- IEEE arithmetic the compiler never fuses -----------------------------
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
// GLSL max(0, v) = (0 < v) ? v : 0.
__device__ __forceinline__ float max0(float v) { return (0.0f < v) ? v : 0.0f; }
// GLSL clamp(v, 0, 1).
__device__ __forceinline__ float saturate01(float v) {
  const float m = (v < 0.0f) ? 0.0f : v;
  return (1.0f < m) ? 1.0f : m;
}

// ---- the source term -----------------------------------------------------------
__device__ __forceinline__ float add_sources(float d, int gx, int gy, const StepArgs& a,
                                             uint32_t mask) {
#pragma unroll
  for (int k = 0; k < TWS_MAX_SOURCES; ++k) {
    if (!((mask >> k) & 1u)) continue;
    const DevSource& s = a.src[k];
    if (gx < s.bx0 || gx > s.bx1 || gy < s.by0 || gy > s.by1) continue;
    if (s.kind == TWS_SOURCE_DISK) {
      const long long dx = gx - s.icx, dy = gy - s.icy;
      if (dx * dx + dy * dy <= (long long)s.ir * s.ir) d = fadd(d, s.rate);
    } else {
      const float tx = fsub(s.cx, (float)gx), ty = fsub(s.cy, (float)gy);
      const float q = fdiv(fadd(fmul(tx, tx), fmul(ty, ty)), s.radius);
      const float inc = fmul(saturate01(fsub(1.0f, q)), s.rate);
      if (inc != 0.0f) d = fadd(d, inc);
    }
  }
  return d;
}


}  // namespace tws
