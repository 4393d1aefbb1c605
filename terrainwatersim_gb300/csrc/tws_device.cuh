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
// The same max(0, v) in one min/max instruction: max.f32 returns the other
// operand for a NaN, and fmaxf(-0, +0) is +0 on sm_103a (measured), so the
// result is the one of max0 for every v.  The GPU tests check it bit for bit
// against the oracle, signed zeros included.
__device__ __forceinline__ float max0_fast(float v) { return fmaxf(v, 0.0f); }
// Divide for the outflow scaling: the dry case (d = +-0, total > 0) is
// d / total = d exactly, which skips the divide for the common dry cell.
__device__ __forceinline__ float scale_factor(float d, float total) {
  return d == 0.0f ? d : fdiv(d, total);
}

// ---- packed pairs (sm_100 and later: add/sub/mul.rn.f32x2) ---------------------
// Each lane is the IEEE round-to-nearest result of its own operands, so one
// pair operation equals two of the scalar helpers above, in half the issue
// slots.  One rule: never feed an fmul2 result into fadd2 or fsub2.  The
// assembler contracts that pair into a packed fused multiply-add despite the
// .rn modifiers and --fmad=false (measured on sm_103a: about half the results
// then differ in the last bit); add packed products with the scalar fadd.
#define TWS_F32X2_OP(name, op)                                                         \
  __device__ __forceinline__ float2 name(float2 a, float2 b) {                        \
    float2 r;                                                                          \
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"                                               \
        "mov.b64 ra, {%2, %3};\n\t"                                                    \
        "mov.b64 rb, {%4, %5};\n\t" op                                                 \
        " rd, ra, rb;\n\t"                                                             \
        "mov.b64 {%0, %1}, rd;\n\t}"                                                   \
        : "=f"(r.x), "=f"(r.y)                                                         \
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                     \
    return r;                                                                          \
  }
TWS_F32X2_OP(fadd2, "add.rn.f32x2")
TWS_F32X2_OP(fsub2, "sub.rn.f32x2")
TWS_F32X2_OP(fmul2, "mul.rn.f32x2")
#undef TWS_F32X2_OP

// F16 storage rounding: the value the next step will read back.
__device__ __forceinline__ float quantize_f16(float v, float scale, float inv_scale) {
  const float s = fminf(fmul(v, scale), 65504.0f);
  return fmul(__half2float(__float2half_rn(s)), inv_scale);
}
// The pair form: one saturating conversion (cvt.rn.satfinite.f16x2.f32) in
// place of min(s, 65504) and a round-to-nearest conversion.  The two agree for
// every input but NaN, which an outflow never is: values of 65520 and above,
// which round to infinity, saturate to 65504 as the clamp gives.
__device__ __forceinline__ float2 quantize_f16x2(float2 v, float2 scale, float2 inv_scale) {
  const float2 s = fmul2(v, scale);
  uint32_t packed;
  asm("cvt.rn.satfinite.f16x2.f32 %0, %1, %2;" : "=r"(packed) : "f"(s.y), "f"(s.x));
  return fmul2(__half22float2(*reinterpret_cast<const __half2*>(&packed)), inv_scale);
}

// GLSL clamp(v, 0, 1).
__device__ __forceinline__ float saturate01(float v) {
  const float m = (v < 0.0f) ? 0.0f : v;
  return (1.0f < m) ? 1.0f : m;
}

// ---- the source term -----------------------------------------------------------
// The integer hash "lowbias32" (C. Wellons, hash-prospector: xorshift-multiply,
// constants 0x7feb352d and 0x846ca68b).
__device__ __forceinline__ uint32_t rain_hash32(uint32_t v) {
  v ^= v >> 16;
  v *= 0x7feb352du;
  v ^= v >> 15;
  v *= 0x846ca68bu;
  v ^= v >> 16;
  return v;
}

// d + r for the DISK rain, rounded without bias.  Round to nearest alone
// biases a 0.01 m increment by a fixed fraction of an ulp of d (+0.24 ulp on
// 8-16 m, -0.44 on 32-64 m, ...), and the total volume of a long rainy run
// drifts with it (up to about 2e-4 of the rain).  TwoSum (Knuth) gives the
// exact rounding error e of s = d + r; s moves one ulp toward d + r when
// u * |step| < |e|, with u in [0, 1) a hash of the cell and the bits of d.
// The expected result is d + r exactly, the run stays deterministic, and
// every operation is exact or IEEE round-to-nearest, as in the oracle.
__device__ __forceinline__ float add_rain(float d, float r, int x, int y) {
  const float s = fadd(d, r);
  const float bp = fsub(s, d);
  const float e = fadd(fsub(d, fsub(s, bp)), fsub(r, bp));
  if (e == 0.0f) return s;
  const uint32_t sb = __float_as_uint(s);
  const float next = __uint_as_float(((s > 0.0f) == (e > 0.0f)) ? sb + 1u : sb - 1u);
  const float step = fsub(next, s);
  const uint32_t h = rain_hash32(__float_as_uint(d) ^
                                 rain_hash32((uint32_t)x ^ rain_hash32((uint32_t)y)));
  const float u = fmul(__uint2float_rn(h >> 8), 0x1p-24f);
  return (fmul(u, fabsf(step)) < fabsf(e)) ? next : s;
}

// Not inlined: only tiles that a source touches call it, and an inlined copy
// in every unrolled cell loop of the tile kernels would multiply their code
// size past the instruction cache.
static __device__ __noinline__ float add_sources(float d, int gx, int gy, const StepArgs& a,
                                                 uint32_t mask) {
#pragma unroll
  for (int k = 0; k < TWS_MAX_SOURCES; ++k) {
    if (!((mask >> k) & 1u)) continue;
    const DevSource& s = a.src[k];
    if (gx < s.bx0 || gx > s.bx1 || gy < s.by0 || gy > s.by1) continue;
    if (s.kind == TWS_SOURCE_DISK) {
      const long long dx = gx - s.icx, dy = gy - s.icy;
      if (dx * dx + dy * dy <= (long long)s.ir * s.ir) d = add_rain(d, s.rate, gx, gy);
    } else {
      const float tx = fsub(s.cx, (float)gx), ty = fsub(s.cy, (float)gy);
      const float q = fdiv(fadd(fmul(tx, tx), fmul(ty, ty)), s.radius);
      const float inc = fmul(saturate01(fsub(1.0f, q)), s.rate);
      if (inc != 0.0f) d = fadd(d, inc);
    }
  }
  return d;
}

// The sources of `mask` at cell (gx, gy), in source order as add_sources
// applies them, without a call: for the compact source passes of the step
// kernels, where one call per cell sat on a launch's critical path (the warps
// under a rain disk were the slowest of a launch) and the saved registers
// around a call would cost the unrolled code around it.
__device__ __forceinline__ float add_sources_inline(float d, int gx, int gy, const StepArgs& a,
                                                    uint32_t mask) {
#pragma unroll 1
  for (int k = 0; k < a.nsrc; ++k) {
    if (!((mask >> k) & 1u)) continue;
    const DevSource& s = a.src[k];
    if (gx < s.bx0 || gx > s.bx1 || gy < s.by0 || gy > s.by1) continue;
    if (s.kind == TWS_SOURCE_DISK) {
      const long long dx = gx - s.icx, dy = gy - s.icy;
      if (dx * dx + dy * dy <= (long long)s.ir * s.ir) d = add_rain(d, s.rate, gx, gy);
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
