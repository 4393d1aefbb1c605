// tws_stream.cu -- the one-step (K = 1) kernel in register-streaming form.
//
// Same arithmetic as the tiled kernel (flowUpdate.comp:34-62 then
// flowApply.comp:32-52, fused, bit-identical to the FP32 transcription), but
// organised so that each cell costs few instructions: a warp owns a strip of
// 30 output columns (32 flux columns: the strip plus one halo column on each
// side) and walks down RY rows of it.  Each lane keeps a rolling window of
// surface heights h = d + b and of new outflows in registers; the x
// neighbours come from the adjacent lanes by warp shuffle (the two halo lanes
// fetch one extra column each), the y neighbours from the window.  Loads of
// row r + 2 are issued while row r is computed (coalesced 4-byte loads of b
// and d, one 16-byte load of the cell's flux record), and there is no shared
// memory and no block barrier.
//
// Per row a lane computes the new outflow of its cell (flux halo included) and,
// one row behind, the depth and flow vector of the cell above; the outputs of
// lanes 1..30 are stored.

#include "tws_device.cuh"
#include "tws_internal.h"

namespace tws {
namespace {

constexpr int kStreamWarps = 4;
constexpr int kStreamThreads = 32 * kStreamWarps;
constexpr int kStrip = 30;  // output columns per warp
constexpr int kStreamMinBlocks = 8;  // 32 warps per SM: at most 64 registers a thread

struct RowIn {
  float b, d;    // own column
  float eb, ed;  // extra column: lane 0 -> x0 - 2, lane 31 -> x0 + 31
};

template <bool INTERIOR>
__device__ __forceinline__ RowIn load_row(const float* __restrict__ b, const float* __restrict__ d,
                                          int pitch, int W, int H, int gx, int ex, int r,
                                          bool edge_lane) {
  RowIn o{0.0f, 0.0f, 0.0f, 0.0f};
  if (INTERIOR) {
    const size_t row = (size_t)r * pitch;
    o.b = __ldg(b + row + gx);
    o.d = __ldg(d + row + gx);
    if (edge_lane) {
      o.eb = __ldg(b + row + ex);
      o.ed = __ldg(d + row + ex);
    }
  } else if (r >= 0 && r < H) {
    const size_t row = (size_t)r * pitch;
    if (gx >= 0 && gx < W) {
      o.b = __ldg(b + row + gx);
      o.d = __ldg(d + row + gx);
    }
    if (edge_lane && ex >= 0 && ex < W) {
      o.eb = __ldg(b + row + ex);
      o.ed = __ldg(d + row + ex);
    }
  }
  return o;
}

template <bool F16>
__device__ __forceinline__ float4 load_flux(const void* __restrict__ f, size_t g, float inv_scale) {
  if (F16) {
    const uint2 raw = __ldg(reinterpret_cast<const uint2*>(f) + g);
    const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&raw.x));
    const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&raw.y));
    return make_float4(fmul(lo.x, inv_scale), fmul(lo.y, inv_scale), fmul(hi.x, inv_scale),
                       fmul(hi.y, inv_scale));
  }
  return __ldg(reinterpret_cast<const float4*>(f) + g);
}

__device__ __forceinline__ float quantize_half(float v, float scale, float inv_scale) {
  const float s = fminf(fmul(v, scale), 65504.0f);
  return fmul(__half2float(__float2half_rn(s)), inv_scale);
}

template <bool INTERIOR, bool F16, int RY>
__device__ __forceinline__ void stream_unit(const StepArgs& a, const float* __restrict__ b,
                                            const float* __restrict__ d,
                                            const void* __restrict__ f, int x0, int y0,
                                            uint32_t mask) {
  const int lane = threadIdx.x & 31;
  const int W = a.W, H = a.H, pitch = a.pitch;
  const int gx = x0 - 1 + lane;                 // this lane's flux column
  const bool edge_lane = lane == 0 || lane == 31;
  const int ex = lane == 0 ? x0 - 2 : x0 + 31;  // extra column of the halo lanes
  const bool col_in = INTERIOR || (gx >= 0 && gx < W);
  const bool ecol_in = INTERIOR || (ex >= 0 && ex < W);
  const bool out_lane = lane >= 1 && lane <= kStrip && (INTERIOR || gx < W);

  auto with_sources = [&](float dv, int x, int r, bool in) -> float {
    return (mask && in && r >= 0 && r < H) ? add_sources_inline(dv, x, r, a, mask) : dv;
  };

  // Window: rows r-1, r, r+1 of h; d of rows r-1, r; new outflow of r-1, r.
  RowIn pm1 = load_row<INTERIOR>(b, d, pitch, W, H, gx, ex, y0 - 2, edge_lane);
  RowIn p0 = load_row<INTERIOR>(b, d, pitch, W, H, gx, ex, y0 - 1, edge_lane);
  RowIn nxt = load_row<INTERIOR>(b, d, pitch, W, H, gx, ex, y0, edge_lane);
  float d_m1 = with_sources(pm1.d, gx, y0 - 2, col_in);
  float h_m1 = fadd(d_m1, pm1.b);
  float d_0 = with_sources(p0.d, gx, y0 - 1, col_in);
  float h_0 = fadd(d_0, p0.b);
  float he_0 = fadd(with_sources(p0.ed, ex, y0 - 1, ecol_in), p0.eb);
  float4 f_cur = make_float4(0.f, 0.f, 0.f, 0.f);
  {
    const int r = y0 - 1;
    if (INTERIOR || (col_in && r >= 0 && r < H))
      f_cur = load_flux<F16>(f, (size_t)r * pitch + gx, a.flux_inv_scale);
  }
  float4 f_m1 = make_float4(0.f, 0.f, 0.f, 0.f);
  float fz_m2 = 0.0f;
  d_m1 = 0.0f;

#pragma unroll 1
  for (int i = y0 - 1; i <= y0 + RY; ++i) {
    // row i + 1 arrives (sources applied), loads of row i + 2 go out
    const int r1 = i + 1;
    const float d_p1 = with_sources(nxt.d, gx, r1, col_in);
    const float h_p1 = fadd(d_p1, nxt.b);
    const float he_p1 = fadd(with_sources(nxt.ed, ex, r1, ecol_in), nxt.eb);
    // (rows up to y0 + RY + 1 are needed; an interior unit has them all in the grid)
    if (i + 2 <= y0 + RY + 1) nxt = load_row<INTERIOR>(b, d, pitch, W, H, gx, ex, i + 2, edge_lane);
    float4 f_nxt = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i + 1 <= y0 + RY && (INTERIOR || (col_in && r1 < H)))
      f_nxt = load_flux<F16>(f, (size_t)r1 * pitch + gx, a.flux_inv_scale);

    // new outflow of row i, flowUpdate.comp:34-62
    float hx1 = __shfl_down_sync(0xffffffffu, h_0, 1);
    float hx0 = __shfl_up_sync(0xffffffffu, h_0, 1);
    if (lane == 31) hx1 = he_0;
    if (lane == 0) hx0 = he_0;
    float4 nf = make_float4(0.f, 0.f, 0.f, 0.f);
    if (INTERIOR || (col_in && i >= 0 && i < H)) {
      nf.x = max0(fadd(fmul(f_cur.x, a.kf), fmul(fsub(h_0, hx1), a.ka)));
      nf.y = max0(fadd(fmul(f_cur.y, a.kf), fmul(fsub(h_0, hx0), a.ka)));
      nf.z = max0(fadd(fmul(f_cur.z, a.kf), fmul(fsub(h_0, h_p1), a.ka)));
      nf.w = max0(fadd(fmul(f_cur.w, a.kf), fmul(fsub(h_0, h_m1), a.ka)));
      if (!INTERIOR && a.closed) {
        if (gx + 1 >= W) nf.x = 0.0f;
        if (gx == 0) nf.y = 0.0f;
        if (i + 1 >= H) nf.z = 0.0f;
        if (i == 0) nf.w = 0.0f;
      }
      const float total = fmul(fadd(fadd(fadd(nf.x, nf.y), nf.z), nf.w), a.c);
      if (total > d_0) {
        const float sc = fdiv(d_0, total);
        nf.x = fmul(nf.x, sc);
        nf.y = fmul(nf.y, sc);
        nf.z = fmul(nf.z, sc);
        nf.w = fmul(nf.w, sc);
      }
      if (F16) {
        nf.x = quantize_half(nf.x, a.flux_scale, a.flux_inv_scale);
        nf.y = quantize_half(nf.y, a.flux_scale, a.flux_inv_scale);
        nf.z = quantize_half(nf.z, a.flux_scale, a.flux_inv_scale);
        nf.w = quantize_half(nf.w, a.flux_scale, a.flux_inv_scale);
      }
    }

    // depth and flow vector of row i - 1, flowApply.comp:32-52
    const float X1 = __shfl_down_sync(0xffffffffu, f_m1.y, 1);
    const float X0 = __shfl_up_sync(0xffffffffu, f_m1.x, 1);
    const int ra = i - 1;
    if (ra >= y0 && out_lane && (INTERIOR || ra < H)) {
      const float Y1 = nf.w, Y0 = fz_m2;
      const float in = fadd(fadd(fadd(X1, X0), Y1), Y0);
      const float out = fadd(fadd(fadd(f_m1.x, f_m1.y), f_m1.z), f_m1.w);
      const float dn = max0(fadd(d_m1, fmul(fsub(in, out), a.c)));
      const size_t g = (size_t)ra * pitch + gx;
      a.d_out[g] = dn;
      if (F16) {
        const __half2 lo = __floats2half2_rn(fmul(f_m1.x, a.flux_scale), fmul(f_m1.y, a.flux_scale));
        const __half2 hi = __floats2half2_rn(fmul(f_m1.z, a.flux_scale), fmul(f_m1.w, a.flux_scale));
        uint2 packed;
        packed.x = *reinterpret_cast<const uint32_t*>(&lo);
        packed.y = *reinterpret_cast<const uint32_t*>(&hi);
        reinterpret_cast<uint2*>(a.f_out)[g] = packed;
      } else {
        reinterpret_cast<float4*>(a.f_out)[g] = f_m1;
      }
      a.v_out[g] = make_float2(fsub(fsub(X1, f_m1.x), fsub(X0, f_m1.y)),
                               fsub(fsub(Y1, f_m1.z), fsub(Y0, f_m1.w)));
    }

    // rotate the window
    fz_m2 = f_m1.z;
    f_m1 = nf;
    f_cur = f_nxt;
    h_m1 = h_0;
    h_0 = h_p1;
    he_0 = he_p1;
    d_m1 = d_0;
    d_0 = d_p1;
  }
}

template <bool F16, int RY>
__global__ void __launch_bounds__(kStreamThreads, kStreamMinBlocks)
    stream_kernel(const float* __restrict__ b, const float* __restrict__ d,
                  const void* __restrict__ f, const __grid_constant__ StepArgs a) {
  const int strips = (a.W + kStrip - 1) / kStrip;
  const int chunks = (a.H + RY - 1) / RY;
  const int unit = blockIdx.x * kStreamWarps + (threadIdx.x >> 5);
  if (unit >= strips * chunks) return;
  const int x0 = (unit % strips) * kStrip;
  const int y0 = (unit / strips) * RY;

  uint32_t mask = 0;
#pragma unroll
  for (int k = 0; k < TWS_MAX_SOURCES; ++k) {
    if (k < a.nsrc) {
      const DevSource& s = a.src[k];
      if (s.bx1 >= x0 - 2 && s.bx0 <= x0 + 31 && s.by1 >= y0 - 2 && s.by0 <= y0 + RY + 1)
        mask |= 1u << k;
    }
  }
  const bool interior = x0 - 2 >= 0 && x0 + 31 < a.W && y0 - 2 >= 0 && y0 + RY + 1 < a.H;
  if (interior)
    stream_unit<true, F16, RY>(a, b, d, f, x0, y0, mask);
  else
    stream_unit<false, F16, RY>(a, b, d, f, x0, y0, mask);
}

}  // namespace

const void* stream_kernel_fn(int ry, int flux_storage) {
  const bool f16 = flux_storage == TWS_FLUX_F16;
  switch (ry) {
    case 32: return f16 ? (const void*)&stream_kernel<true, 32> : (const void*)&stream_kernel<false, 32>;
    case 64: return f16 ? (const void*)&stream_kernel<true, 64> : (const void*)&stream_kernel<false, 64>;
    case 128: return f16 ? (const void*)&stream_kernel<true, 128> : (const void*)&stream_kernel<false, 128>;
    default: return nullptr;
  }
}

cudaError_t launch_stream_step(int ry, int flux_storage, const float* b, const float* d,
                               const void* f, const StepArgs& a, cudaStream_t s) {
  const void* fn = stream_kernel_fn(ry, flux_storage);
  if (!fn) return cudaErrorInvalidValue;
  const long long strips = (a.W + kStrip - 1) / kStrip, chunks = (a.H + ry - 1) / ry;
  const long long blocks = (strips * chunks + kStreamWarps - 1) / kStreamWarps;
  using Fn = void (*)(const float*, const float*, const void*, StepArgs);
  reinterpret_cast<Fn>(const_cast<void*>(fn))<<<(unsigned)blocks, kStreamThreads, 0, s>>>(b, d, f, a);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tws
