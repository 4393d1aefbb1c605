// tws_step.cu -- the fused virtual-pipe step kernel for sm_103a.
//
// One launch advances a grid by K steps (K = 1: the plain kernel; K > 1:
// temporal blocking).  Per step and per cell it computes, in the reference's
// operation order:
//   source term              waterBrush.comp:26-28 / the benchmark's rain disk
//   outflow flux + scaling   flowUpdate.comp:34-62
//   depth update, flow map   flowApply.comp:32-52
// The two reference dispatches (Terrain.cpp:253-265) become one kernel: a CTA
// owns a TX x TY tile of output cells, loads b and d with a 2K-cell halo and
// the flux box into shared memory with TMA (cp.async.bulk.tensor, completion
// on an mbarrier), recomputes the halo fluxes it needs, and writes d, f and
// the flow map of its tile once.  Halo cells are recomputed redundantly by
// neighbouring CTAs, so there is no inter-CTA dependency inside a launch.
// Two layouts: the separate one (flux box = the (2K-1)-cell halo, 2-D loops,
// process_tile) and the unified one (flux box = the b/d box, flat loops over
// one index, flux in channel planes, packed f32x2 arithmetic:
// process_tile_flat), which the default variants use.
//
// STAGES = 2 makes the CTAs persistent: each walks the tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... and keeps the TMA load of its next
// tile in flight in a second buffer while it computes the current one, so
// HBM reads continue through the compute phases.  STAGES = 1 launches one CTA
// per tile.
//
// Arithmetic is IEEE round-to-nearest with no contraction (__fmul_rn etc.),
// so the result is bit-identical to the FP32 CPU transcription of the shaders.
//
// HBM layout (per grid): b, d[2] float with a row pitch that is a multiple of
// 32 elements; f[2] float4 (or 4 x half) per cell, same pitch; v float2.

#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <type_traits>

#include "tws_device.cuh"
#include "tws_internal.h"

namespace tws {
namespace {

constexpr int kThreads = 256;

// ---- shared memory / TMA / mbarrier primitives -----------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Programmatic dependent launch.  A step launch may be scheduled while the
// previous launch on the stream is still finishing; it waits here, before
// its first global-memory access, until that launch has completed and its
// writes are visible (a hardware wait that ends when the previous grid does).
// Having passed it, the CTA lets the next launch be scheduled in turn.
__device__ __forceinline__ void wait_previous_launch() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void allow_next_launch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
// Orders this thread's view of earlier generic-proxy shared-memory accesses
// (made visible to it by __syncthreads) before a following TMA write.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int c0, int c1,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int c0, int c1,
                                            int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

// The dynamic shared memory base rounded up to 128 bytes (TMA destinations),
// by pointer arithmetic on the shared array so the compiler keeps every access
// derived from it in the shared window (LDS/STS, not generic loads).
__device__ __forceinline__ unsigned char* align_smem(unsigned char* raw) {
  return raw + ((128u - (smem_u32(raw) & 127u)) & 127u);
}

// Bounded wait on phase `parity`: gives up after `limit` SM clocks (by default
// about two seconds; a tile load takes microseconds).  On time-out: record
// the error, wait once more (bounded) for the barrier, report false.
//
// What the second wait can and cannot ensure: a copy that lands late but
// lands completes the barrier, so the CTA leaves only after it.  A copy that
// never completes cannot be observed or cancelled from the SM; the CTA then
// leaves after the second limit with that copy still pending.  Only a fault
// of the memory system can cause that, and the grid's error word reports the
// time-out either way, after which the host reloads the state.  The test
// hook (tws_test_drop_tile_loads) arms the barrier without issuing any copy,
// so the tested path has nothing in flight.
__device__ bool wait_bounded(uint64_t* bar, uint32_t parity, int* err, long long limit) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > limit) {
      atomicExch(err, kDevErrWaitTimeout);
      const long long t1 = clock64();
      while (!mbar_try_wait(bar, parity) && clock64() - t1 < limit) {
      }
      return false;
    }
  }
  return true;
}

// ---- tile geometry -----------------------------------------------------------
__host__ __device__ constexpr size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// UNI = false: the flux box is the (2K-1)-cell halo the K steps need.
// UNI = true (unified layout): the flux box is the b/d box itself, so b, d,
// h and f share one row stride and one index per cell; interior tiles then
// walk their rings as flat runs of that index (process_tile_flat).  It loads
// a few more flux records per tile (served from L2).
template <int K, int TX, int TY, bool F16, int STAGES, bool UNI = false>
struct Tile {
  static constexpr int HX = (2 * K + 3) / 4 * 4;  // x halo of b/d, whole 16-byte units
  static constexpr int HY = 2 * K;                // y halo of b/d
  static constexpr int BW = TX + 2 * HX, BH = TY + 2 * HY;
  static constexpr int RF = 2 * K - 1;  // flux halo the K steps need
  // flux box: origin (x0 - FOX, y0 - FOY), FW x FH cells
  static constexpr int FOX = UNI ? HX : RF, FOY = UNI ? HY : RF;
  static constexpr int FW = UNI ? BW : TX + 2 * RF, FH = UNI ? BH : TY + 2 * RF;
  // F16 staging: whole cell pairs from SOFF cells before the flux box (the box
  // origin must be an even cell; x0 - 2K is, and so is x0 - HX)
  static constexpr int SOFF = UNI ? 0 : 1;
  static constexpr int SW = FW + 2 * SOFF;  // staging width in cells
  static constexpr int NB = BW * BH, NF = FW * FH;
  // flux-box index of the cell at flux-ring coordinates (fi, fj), whose
  // origin is (x0 - RF, y0 - RF)
  static constexpr int FOFF = (FOY - RF) * FW + (FOX - RF);
  // One stage = what TMA writes for one tile: b, d and the flux box (float4
  // records for F32 storage, the raw halves for F16 storage).  In the unified
  // layout the flux region always has room for NF float records: the tile
  // code keeps the flux there as four channel planes of NB floats
  // (process_tile_flat).
  static constexpr size_t ST_B = 0;
  static constexpr size_t ST_D = align_up((size_t)NB * 4, 128);
  static constexpr size_t ST_F = align_up(ST_D + (size_t)NB * 4, 128);
  static constexpr size_t ST_BYTES =
      align_up(ST_F + ((F16 && !UNI) ? (size_t)SW * FH * 8 : (size_t)NF * 16), 128);
  // Working arrays shared by all stages: surface height h, and (F16 storage,
  // separate layout) the float4 copy of the flux.  With one step per launch
  // the terrain is not needed once h = d + b is formed, so h overwrites b in
  // place (H_ALIAS) and the tile needs less shared memory (more CTAs per SM).
  static constexpr bool H_ALIAS = (K == 1);
  static constexpr size_t OFF_H = STAGES * ST_BYTES;
  static constexpr size_t OFF_WORK = align_up(OFF_H + (H_ALIAS ? 0 : (size_t)NB * 4), 128);
  static constexpr size_t OFF_BAR =
      align_up(OFF_WORK + ((F16 && !UNI) ? (size_t)NF * 16 : 0), 128);
  static constexpr size_t SMEM = OFF_BAR + 8 * STAGES + 128;  // + slack to align the base
  static constexpr uint32_t TX_BYTES = (uint32_t)(2 * NB * 4 + (F16 ? SW * FH * 8 : NF * 16));
};

// The three TMA loads of the tile at (x0, y0) into one stage buffer.
// `drop` (normally 0) is the test hook of tws_test_drop_tile_loads: the
// barrier is armed for the tile's bytes but no copy is issued, so its wait
// runs out with nothing in flight.
template <class T, bool F16>
__device__ __forceinline__ void issue_tile(unsigned char* st, uint64_t* bar,
                                           const CUtensorMap* tm_b, const CUtensorMap* tm_d,
                                           const CUtensorMap* tm_f, int x0, int y0,
                                           int drop = 0) {
  mbar_expect_tx(bar, T::TX_BYTES);
  if (drop) return;
  tma_load_2d(st + T::ST_B, tm_b, x0 - T::HX, y0 - T::HY, bar);
  tma_load_2d(st + T::ST_D, tm_d, x0 - T::HX, y0 - T::HY, bar);
  if (F16) {
    // cell pairs; x0 - FOX - SOFF is even
    tma_load_3d(st + T::ST_F, tm_f, 0, (x0 - T::FOX - T::SOFF) / 2, y0 - T::FOY, bar);
  } else {
    tma_load_3d(st + T::ST_F, tm_f, 0, x0 - T::FOX, y0 - T::FOY, bar);
  }
}

// K steps of one tile of the separate layout whose loads have landed in (sb,
// sd, sf-or-staging).  INTERIOR: the tile's whole b/d box lies inside the
// grid, so no cell it computes is off the grid or on the border (no bounds or
// wall checks).
template <int K, int TX, int TY, bool F16, int STAGES, bool INTERIOR>
__device__ __forceinline__ void process_tile(const StepArgs& a, float* __restrict__ d_out,
                                             void* __restrict__ f_out, float2* __restrict__ v_out,
                                             int x0, int y0, uint32_t mask, float* sb, float* sd,
                                             float* sh, float4* sf, const unsigned char* staging) {
  using T = Tile<K, TX, TY, F16, STAGES, false>;
  const int tid = threadIdx.x;
  // The per-grid scalars, read once (in the batched kernel `a` lives in
  // global memory; in registers the loops below do not reload them).
  const int W = a.W, H = a.H;
  const float kf = a.kf, ka = a.ka, cc = a.c;
  const float fscale = a.flux_scale, finv = a.flux_inv_scale;
  const bool closed = a.closed != 0;

  // Phase 0: first step's sources, surface height h = d + b (flowUpdate.comp:34).
  // The sources are a compact pass of their own (only tiles a source reaches
  // make it), with the same cells per thread as the loop after it.
  if (mask) {
#pragma unroll 1
    for (int idx = tid; idx < T::NB; idx += kThreads) {
      const int i = idx / T::BW, j = idx - (idx / T::BW) * T::BW;
      const int gx = x0 - T::HX + j, gy = y0 - T::HY + i;
      if (INTERIOR || (gx >= 0 && gx < W && gy >= 0 && gy < H))
        sd[idx] = add_sources_inline(sd[idx], gx, gy, a, mask);
    }
  }
  for (int idx = tid; idx < T::NB; idx += kThreads) sh[idx] = fadd(sd[idx], sb[idx]);
  if (F16) {
    const __half2* st = reinterpret_cast<const __half2*>(staging);
    for (int idx = tid; idx < T::NF; idx += kThreads) {
      const int i = idx / T::FW, j = idx - (idx / T::FW) * T::FW;
      const int s = i * T::SW + j + T::SOFF;
      const float2 lo = __half22float2(st[2 * s]), hi = __half22float2(st[2 * s + 1]);
      sf[idx] = make_float4(fmul(lo.x, finv), fmul(lo.y, finv), fmul(hi.x, finv),
                            fmul(hi.y, finv));
    }
  }
  __syncthreads();

#pragma unroll
  for (int s = 0; s < K; ++s) {
    const int rf = T::RF - 2 * s;  // ring of flux computed in this step
    const int rd = rf - 1;         // ring of depth computed in this step

    // Phase A: outflow flux with non-negativity scaling, flowUpdate.comp:34-62.
    {
      const int RW = TX + 2 * rf, RH = TY + 2 * rf;
      for (int idx = tid; idx < RW * RH; idx += kThreads) {
        const int i = idx / RW, j = idx - (idx / RW) * RW;
        const int fi = T::RF - rf + i, fj = T::RF - rf + j;
        const int gx = x0 - T::RF + fj, gy = y0 - T::RF + fi;
        if (!INTERIOR && (gx < 0 || gx >= W || gy < 0 || gy >= H)) continue;
        const int bidx = (fi + T::HY - T::RF) * T::BW + (fj + T::HX - T::RF);
        const float hc = sh[bidx];
        const float ex1 = fsub(hc, sh[bidx + 1]);
        const float ex0 = fsub(hc, sh[bidx - 1]);
        const float ey1 = fsub(hc, sh[bidx + T::BW]);
        const float ey0 = fsub(hc, sh[bidx - T::BW]);
        const float dc = sd[bidx];
        const int fidx = fi * T::FW + fj + T::FOFF;
        const float4 fo = sf[fidx];
        float4 nf;
        nf.x = max0(fadd(fmul(fo.x, kf), fmul(ex1, ka)));
        nf.y = max0(fadd(fmul(fo.y, kf), fmul(ex0, ka)));
        nf.z = max0(fadd(fmul(fo.z, kf), fmul(ey1, ka)));
        nf.w = max0(fadd(fmul(fo.w, kf), fmul(ey0, ka)));
        if (!INTERIOR && closed) {
          if (gx + 1 >= W) nf.x = 0.0f;
          if (gx == 0) nf.y = 0.0f;
          if (gy + 1 >= H) nf.z = 0.0f;
          if (gy == 0) nf.w = 0.0f;
        }
        const float total = fmul(fadd(fadd(fadd(nf.x, nf.y), nf.z), nf.w), cc);
        if (total > dc) {
          const float sc = scale_factor(dc, total);
          nf.x = fmul(nf.x, sc);
          nf.y = fmul(nf.y, sc);
          nf.z = fmul(nf.z, sc);
          nf.w = fmul(nf.w, sc);
        }
        if (F16) {
          nf.x = quantize_f16(nf.x, fscale, finv);
          nf.y = quantize_f16(nf.y, fscale, finv);
          nf.z = quantize_f16(nf.z, fscale, finv);
          nf.w = quantize_f16(nf.w, fscale, finv);
        }
        sf[fidx] = nf;
      }
    }
    __syncthreads();

    // Phase B: depth update and flow vector, flowApply.comp:32-52.
    {
      const int RW = TX + 2 * rd, RH = TY + 2 * rd;
      for (int idx = tid; idx < RW * RH; idx += kThreads) {
        const int i = idx / RW, j = idx - (idx / RW) * RW;
        const int fi = T::RF - rd + i, fj = T::RF - rd + j;
        const int gx = x0 - T::RF + fj, gy = y0 - T::RF + fi;
        if (!INTERIOR && (gx < 0 || gx >= W || gy < 0 || gy >= H)) continue;
        const int fidx = fi * T::FW + fj + T::FOFF;
        const float4 fc = sf[fidx];
        const float X1 = sf[fidx + 1].y;      // -x outflow of the +x neighbour
        const float X0 = sf[fidx - 1].x;      // +x outflow of the -x neighbour
        const float Y1 = sf[fidx + T::FW].w;  // -y outflow of the +y neighbour
        const float Y0 = sf[fidx - T::FW].z;  // +y outflow of the -y neighbour
        const int bidx = (fi + T::HY - T::RF) * T::BW + (fj + T::HX - T::RF);
        const float in = fadd(fadd(fadd(X1, X0), Y1), Y0);
        const float out = fadd(fadd(fadd(fc.x, fc.y), fc.z), fc.w);
        const float dn = max0(fadd(sd[bidx], fmul(fsub(in, out), cc)));
        if (s == K - 1) {
          const size_t g = (size_t)gy * a.pitch + gx;
          d_out[g] = dn;
          if (F16) {
            const __half2 lo =
                __floats2half2_rn(fmul(fc.x, fscale), fmul(fc.y, fscale));
            const __half2 hi =
                __floats2half2_rn(fmul(fc.z, fscale), fmul(fc.w, fscale));
            uint2 packed;
            packed.x = *reinterpret_cast<const uint32_t*>(&lo);
            packed.y = *reinterpret_cast<const uint32_t*>(&hi);
            reinterpret_cast<uint2*>(f_out)[g] = packed;
          } else {
            reinterpret_cast<float4*>(f_out)[g] = fc;
          }
          v_out[g] = make_float2(fsub(fsub(X1, fc.x), fsub(X0, fc.y)),
                                   fsub(fsub(Y1, fc.z), fsub(Y0, fc.w)));
        } else {
          sd[bidx] = dn;
          sh[bidx] = fadd(dn, sb[bidx]);
        }
      }
      if (s < K - 1 && mask) {
        // the next step's sources: a compact pass over the same cells per thread
#pragma unroll 1
        for (int idx = tid; idx < RW * RH; idx += kThreads) {
          const int i = idx / RW, j = idx - (idx / RW) * RW;
          const int fi = T::RF - rd + i, fj = T::RF - rd + j;
          const int gx = x0 - T::RF + fj, gy = y0 - T::RF + fi;
          if (!INTERIOR && (gx < 0 || gx >= W || gy < 0 || gy >= H)) continue;
          const int bidx = (fi + T::HY - T::RF) * T::BW + (fj + T::HX - T::RF);
          const float d = add_sources_inline(sd[bidx], gx, gy, a, mask);
          sd[bidx] = d;
          sh[bidx] = fadd(d, sb[bidx]);
        }
      }
    }
    if (s < K - 1) __syncthreads();
  }
}

// Runs body(p) for p = FIRST .. LAST, thread tid taking FIRST + tid,
// FIRST + tid + kThreads, ...: fully unrolled, so every position's shared
// memory address is a constant offset from one register.
// UNROLL = false: an ordinary loop instead (tiles at the grid's edge, which
// are few: their code stays small and out of the instruction cache's way).
template <int FIRST, int LAST, bool UNROLL, class F>
__device__ __forceinline__ void ring_for(int tid, F&& body) {
  if constexpr (UNROLL) {
    constexpr int N = LAST - FIRST + 1;
    constexpr int FULL = N / kThreads, REM = N % kThreads;
#pragma unroll
    for (int it = 0; it < FULL; ++it) body(FIRST + it * kThreads + tid);
    if (REM > 0 && tid < REM) body(FIRST + FULL * kThreads + tid);
  } else {
#pragma unroll 1
    for (int p = FIRST + tid; p <= LAST; p += kThreads) body(p);
  }
}

// K steps of an interior tile in the unified layout: b, d, h and f share the
// box index p = r * BW + c (box row r, column c).  The ring of a phase is
// the box rows and columns [lo, hi); the phase walks the single run of p from
// (lo_r, lo_c) to (hi_r - 1, hi_c - 1), which also covers the wrap-around
// cells between the ring's rows.  Those cells lie outside the ring, so what
// they compute lands only where no later phase reads (the rings shrink by
// two cells per step); their neighbour reads stay inside the box.  The runs
// are compile-time ranges (ring_for), so no 2-D index and no loop counter is
// computed per cell.
//
// The flux is worked on as four channel planes (fx, fy, fz, fw: +x, -x, +y,
// -y outflow).  The depth update reads one channel of each neighbour; from
// planes that is one conflict-free shared-memory wavefront per warp, where a
// float4 record array needs four.  The planes occupy the bytes of the TMA
// flux box, so the first step's outflow pass reads the box (float4 records,
// or the F16 halves) into registers, waits for the whole CTA, then writes the
// planes: no extra shared memory, so as many CTAs fit per SM as before.
//
// The cell arithmetic is process_tile's, with channel pairs in packed f32x2
// operations, so results are identical.
//
// INTERIOR: the box lies inside the grid.  Otherwise (a tile at the grid's
// edge) each visited cell finds its grid coordinates from p: cells off the
// grid keep the zero flux, depth and surface the box loaded with (the
// shaders' out-of-range reads), and closed walls zero the outflow across the
// border, as in process_tile.
template <int K, int TX, int TY, bool F16, int STAGES, bool INTERIOR>
__device__ __forceinline__ void process_tile_flat(const StepArgs& a, float* __restrict__ d_out,
                                                  void* __restrict__ f_out,
                                                  float2* __restrict__ v_out, int x0, int y0,
                                                  uint32_t mask, float* sb, float* sd, float* sh,
                                                  unsigned char* fbox) {
  using T = Tile<K, TX, TY, F16, STAGES, true>;
  constexpr int S = T::BW;
  static_assert((TX * TY) % kThreads == 0, "the output tile is whole rounds of the CTA");
  const int tid = threadIdx.x;
  const float kf = a.kf, ka = a.ka, cc = a.c;
  const float fscale = a.flux_scale, finv = a.flux_inv_scale;
  const float2 kf2 = make_float2(kf, kf), ka2 = make_float2(ka, ka);
  const float2 fscale2 = make_float2(fscale, fscale), finv2 = make_float2(finv, finv);
  const int W = a.W, H = a.H;
  const bool closed = a.closed != 0;
  // grid coordinates of box cell p, and whether it is on the grid
  auto cell = [&](int p, int& gx, int& gy) {
    const int r = p / S;
    gx = x0 - T::HX + (p - r * S);
    gy = y0 - T::HY + r;
    return INTERIOR || (gx >= 0 && gx < W && gy >= 0 && gy < H);
  };
  float* const planes = reinterpret_cast<float*>(fbox);
  float* __restrict__ fx = planes;
  float* __restrict__ fy = planes + T::NB;
  float* __restrict__ fz = planes + 2 * T::NB;
  float* __restrict__ fw = planes + 3 * T::NB;
  // box index of the first and last cell of ring r (r cells beyond the tile)
  constexpr auto first = [](int r) { return (T::HY - r) * S + (T::HX - r); };
  constexpr auto last = [](int r) { return (T::HY + TY + r - 1) * S + (T::HX + TX + r - 1); };

  // Phase 0: first step's sources and h = d + b (flowUpdate.comp:34).  The
  // sources are a compact pass of their own, outside the unrolled runs (only
  // tiles a source reaches make it), over the same cells per thread as the
  // run after it.
  if (mask) {
    ring_for<0, T::NB - 1, false>(tid, [&](int p) {
      int gx, gy;
      if (cell(p, gx, gy)) sd[p] = add_sources_inline(sd[p], gx, gy, a, mask);
    });
  }
  ring_for<0, T::NB - 1, INTERIOR>(tid, [&](int p) { sh[p] = fadd(sd[p], sb[p]); });
  // The flux of cell p as the TMA box holds it (float4 records, or halves).
  auto box_flux = [&](int p) -> float4 {
    if constexpr (F16) {
      const __half2* st = reinterpret_cast<const __half2*>(fbox);
      const float2 lo = fmul2(__half22float2(st[2 * p]), finv2);
      const float2 hi = fmul2(__half22float2(st[2 * p + 1]), finv2);
      return make_float4(lo.x, lo.y, hi.x, hi.y);
    } else {
      return reinterpret_cast<const float4*>(fbox)[p];
    }
  };
  if constexpr (!INTERIOR) {
    // Edge tiles turn the box into planes first (all reads, then all writes:
    // the planes overwrite the box), so that every step reads planes.
    constexpr int F = first(T::RF), N = last(T::RF) - F + 1;
    constexpr int IT = (N + kThreads - 1) / kThreads;
    float4 w[IT];
#pragma unroll
    for (int it = 0; it < IT; ++it)
      if (it * kThreads + tid < N) w[it] = box_flux(F + it * kThreads + tid);
    __syncthreads();
#pragma unroll
    for (int it = 0; it < IT; ++it)
      if (it * kThreads + tid < N) {
        const int p = F + it * kThreads + tid;
        fx[p] = w[it].x;
        fy[p] = w[it].y;
        fz[p] = w[it].z;
        fw[p] = w[it].w;
      }
  }
  __syncthreads();

  // Phase A: outflow flux with non-negativity scaling, flowUpdate.comp:34-62.
  // Channel pairs (+x, -x) and (+y, -y) go through the packed f32x2 ops.
  auto outflow = [&](int p, auto s_) -> float4 {
    constexpr int s = decltype(s_)::value;
    int gx = 0, gy = 0;
    if (!cell(p, gx, gy)) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // stays zero
    const float4 fo =
        (s > 0 || !INTERIOR) ? make_float4(fx[p], fy[p], fz[p], fw[p]) : box_flux(p);
    const float hc = sh[p];
    const float2 hc2 = make_float2(hc, hc);
    const float2 ex = fsub2(hc2, make_float2(sh[p + 1], sh[p - 1]));  // (+x, -x)
    const float2 ey = fsub2(hc2, make_float2(sh[p + S], sh[p - S]));  // (+y, -y)
    const float dc = sd[p];
    // products in pairs, their sums scalar (a packed add of packed products
    // would be contracted to a fused multiply-add)
    const float2 px = fmul2(make_float2(fo.x, fo.y), kf2), qx = fmul2(ex, ka2);
    const float2 py = fmul2(make_float2(fo.z, fo.w), kf2), qy = fmul2(ey, ka2);
    float2 nx = make_float2(max0_fast(fadd(px.x, qx.x)), max0_fast(fadd(px.y, qx.y)));
    float2 ny = make_float2(max0_fast(fadd(py.x, qy.x)), max0_fast(fadd(py.y, qy.y)));
    if (!INTERIOR && closed) {  // no outflow across a closed wall
      if (gx + 1 >= W) nx.x = 0.0f;
      if (gx == 0) nx.y = 0.0f;
      if (gy + 1 >= H) ny.x = 0.0f;
      if (gy == 0) ny.y = 0.0f;
    }
    const float total = fmul(fadd(fadd(fadd(nx.x, nx.y), ny.x), ny.y), cc);
    if (total > dc) {
      const float sc = scale_factor(dc, total);
      const float2 sc2 = make_float2(sc, sc);
      nx = fmul2(nx, sc2);
      ny = fmul2(ny, sc2);
    }
    if (F16) {
      nx = quantize_f16x2(nx, fscale2, finv2);
      ny = quantize_f16x2(ny, fscale2, finv2);
    }
    return make_float4(nx.x, nx.y, ny.x, ny.y);
  };
  auto store = [&](int p, float4 f) {
    fx[p] = f.x;
    fy[p] = f.y;
    fz[p] = f.z;
    fw[p] = f.w;
  };
  // (inflow, outflow) of cell p summed side by side, each in the shader's
  // order: in = ((X1 + X0) + Y1) + Y0 from the neighbours' channels toward p,
  // out = ((fx + fy) + fz) + fw.
  auto in_out = [&](int p, float4 fc) {
    float2 io = fadd2(make_float2(fy[p + 1], fc.x), make_float2(fx[p - 1], fc.y));
    io = fadd2(io, make_float2(fw[p + S], fc.z));
    return fadd2(io, make_float2(fz[p - S], fc.w));
  };
  // Phase B: depth update, flowApply.comp:32-52, and surface height; the next
  // step's sources follow in their own pass (depth_sources).
  auto depth = [&](int p) {
    if constexpr (!INTERIOR) {
      int gx, gy;
      if (!cell(p, gx, gy)) return;  // off the grid: depth and surface stay zero
    }
    const float4 fc = make_float4(fx[p], fy[p], fz[p], fw[p]);
    const float2 io = in_out(p, fc);
    const float dn = max0_fast(fadd(sd[p], fmul(fsub(io.x, io.y), cc)));
    sd[p] = dn;
    sh[p] = fadd(dn, sb[p]);
  };
  auto depth_sources = [&](int p) {
    int gx, gy;
    if (!cell(p, gx, gy)) return;
    const float d = add_sources_inline(sd[p], gx, gy, a, mask);
    sd[p] = d;
    sh[p] = fadd(d, sb[p]);
  };
  // The last step's depth ring is the tile itself: depth, flux and flow map
  // (flowApply.comp:32-52) go out to the grid.
  auto finish = [&]() {
    const size_t pitch = (size_t)a.pitch;
#pragma unroll
    for (int it = 0; it < TX * TY / kThreads; ++it) {
      const int idx = it * kThreads + tid;
      const int i = idx / TX, j = idx % TX;
      if (!INTERIOR && (x0 + j >= W || y0 + i >= H)) continue;  // past the grid's edge
      const int p = (T::HY + i) * S + T::HX + j;
      const float4 fc = make_float4(fx[p], fy[p], fz[p], fw[p]);
      const float X1 = fy[p + 1];  // -x outflow of the +x neighbour
      const float X0 = fx[p - 1];  // +x outflow of the -x neighbour
      const float Y1 = fw[p + S];  // -y outflow of the +y neighbour
      const float Y0 = fz[p - S];  // +y outflow of the -y neighbour
      float2 io = fadd2(make_float2(X1, fc.x), make_float2(X0, fc.y));
      io = fadd2(io, make_float2(Y1, fc.z));
      io = fadd2(io, make_float2(Y0, fc.w));
      const float dn = max0_fast(fadd(sd[p], fmul(fsub(io.x, io.y), cc)));
      const size_t g = (size_t)(y0 + i) * pitch + (size_t)(x0 + j);
      d_out[g] = dn;
      if (F16) {
        const __half2 lo = __float22half2_rn(fmul2(make_float2(fc.x, fc.y), fscale2));
        const __half2 hi = __float22half2_rn(fmul2(make_float2(fc.z, fc.w), fscale2));
        uint2 packed;
        packed.x = *reinterpret_cast<const uint32_t*>(&lo);
        packed.y = *reinterpret_cast<const uint32_t*>(&hi);
        reinterpret_cast<uint2*>(f_out)[g] = packed;
      } else {
        reinterpret_cast<float4*>(f_out)[g] = fc;
      }
      v_out[g] = fsub2(fsub2(make_float2(X1, Y1), make_float2(fc.x, fc.z)),
                       fsub2(make_float2(X0, Y0), make_float2(fc.y, fc.w)));
    }
  };
  // step s computes the flux on ring RF - 2s and the depth on the ring inside it
  auto step = [&](auto s_) {
    constexpr int s = decltype(s_)::value;
    constexpr int rf = T::RF - 2 * s;
    if constexpr (s == 0 && INTERIOR) {
      // the planes overwrite the box: all reads first, then all writes
      constexpr int F = first(rf), N = last(rf) - F + 1;
      constexpr int IT = (N + kThreads - 1) / kThreads;
      float4 r[IT];
#pragma unroll
      for (int it = 0; it < IT; ++it)
        if (it * kThreads + tid < N) r[it] = outflow(F + it * kThreads + tid, s_);
      __syncthreads();
#pragma unroll
      for (int it = 0; it < IT; ++it)
        if (it * kThreads + tid < N) store(F + it * kThreads + tid, r[it]);
    } else {
      ring_for<first(rf), last(rf), INTERIOR>(tid, [&](int p) { store(p, outflow(p, s_)); });
    }
    __syncthreads();
    if constexpr (s < K - 1) {
      ring_for<first(rf - 1), last(rf - 1), INTERIOR>(tid, depth);
      // same cells per thread as the run above: no barrier between the two
      if (mask) ring_for<first(rf - 1), last(rf - 1), false>(tid, depth_sources);
      __syncthreads();
    } else {
      finish();
    }
  };
  step(std::integral_constant<int, 0>{});
  if constexpr (K > 1) step(std::integral_constant<int, 1>{});
  if constexpr (K > 2) step(std::integral_constant<int, 2>{});
  if constexpr (K > 3) step(std::integral_constant<int, 3>{});
  static_assert(K <= 4, "steps per launch");
}

// ---- the kernel --------------------------------------------------------------
template <int K, int TX, int TY, bool F16, int STAGES, bool UNI>
__global__ void __launch_bounds__(kThreads)
    step_kernel(const __grid_constant__ CUtensorMap tm_b, const __grid_constant__ CUtensorMap tm_d,
                const __grid_constant__ CUtensorMap tm_f, const __grid_constant__ StepArgs a) {
  using T = Tile<K, TX, TY, F16, STAGES, UNI>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = align_smem(smem_raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + T::OFF_BAR);

  const int tid = threadIdx.x;
  // One CTA per tile (STAGES == 1) takes its tile from a 2-D grid; the
  // persistent form walks the tiles by a 1-D numbering.
  const int tiles_x = STAGES == 1 ? 1 : (a.W + TX - 1) / TX;
  const int num_tiles = STAGES == 1 ? 1 : tiles_x * ((a.H + TY - 1) / TY);
  const int first = STAGES == 1 ? 0 : (int)blockIdx.x;
  const int stride = STAGES == 1 ? 1 : (int)gridDim.x;
  auto tile_origin = [&](int t, int& x0, int& y0) {
    if (STAGES == 1) {
      x0 = blockIdx.x * TX;
      y0 = blockIdx.y * TY;
    } else {
      x0 = (t % tiles_x) * TX;
      y0 = (t / tiles_x) * TY;
    }
  };

  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  wait_previous_launch();
  allow_next_launch();
  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < STAGES; ++s) {
      const int t = first + s * stride;
      if (t < num_tiles) {
        int tx0, ty0;
        tile_origin(t, tx0, ty0);
        issue_tile<T, F16>(smem + s * T::ST_BYTES, &bars[s], &tm_b, &tm_d, &tm_f, tx0, ty0,
                           a.drop_loads);
      }
    }
  }

  int it = 0;
  for (int t = first; t < num_tiles; t += stride, ++it) {
    const int s = STAGES == 1 ? 0 : it % STAGES;
    const uint32_t parity = (uint32_t)((it / STAGES) & 1);
    unsigned char* st = smem + s * T::ST_BYTES;
    float* sb = reinterpret_cast<float*>(st + T::ST_B);
    float* sd = reinterpret_cast<float*>(st + T::ST_D);
    float* sh = T::H_ALIAS ? sb : reinterpret_cast<float*>(smem + T::OFF_H);
    float4* sf = (F16 && !UNI) ? reinterpret_cast<float4*>(smem + T::OFF_WORK)
                               : reinterpret_cast<float4*>(st + T::ST_F);
    int x0, y0;
    tile_origin(t, x0, y0);

    // Which sources can touch this tile's b/d box.
    uint32_t mask = 0;
    for (int k = 0; k < a.nsrc; ++k) {
      const DevSource& src = a.src[k];
      if (src.bx1 >= x0 - T::HX && src.bx0 < x0 + TX + T::HX && src.by1 >= y0 - T::HY &&
          src.by0 < y0 + TY + T::HY)
        mask |= 1u << k;
    }

    const bool ok = wait_bounded(&bars[s], parity, a.err, a.wait_cycles);
    if (__syncthreads_or(!ok)) {  // every thread leaves together on a time-out
      if (STAGES > 1 && tid == 0) {
        // the loads already issued into the other stages are waited for
        // (bounded) first, so that none is left writing into shared memory
#pragma unroll
        for (int j = 1; j < STAGES; ++j) {
          if (t + j * stride < num_tiles)
            wait_bounded(&bars[(it + j) % STAGES], (uint32_t)(((it + j) / STAGES) & 1), a.err,
                         a.wait_cycles);
        }
      }
      return;
    }

    const bool interior =
        x0 - T::HX >= 0 && y0 - T::HY >= 0 && x0 + TX + T::HX <= a.W && y0 + TY + T::HY <= a.H;
    if constexpr (UNI) {
      if (interior)
        process_tile_flat<K, TX, TY, F16, STAGES, true>(a, a.d_out, a.f_out, a.v_out, x0, y0,
                                                        mask, sb, sd, sh, st + T::ST_F);
      else
        process_tile_flat<K, TX, TY, F16, STAGES, false>(a, a.d_out, a.f_out, a.v_out, x0, y0,
                                                         mask, sb, sd, sh, st + T::ST_F);
    } else if (interior) {
      process_tile<K, TX, TY, F16, STAGES, true>(a, a.d_out, a.f_out, a.v_out, x0, y0, mask,
                                                      sb, sd, sh, sf, st + T::ST_F);
    } else {
      process_tile<K, TX, TY, F16, STAGES, false>(a, a.d_out, a.f_out, a.v_out, x0, y0, mask,
                                                       sb, sd, sh, sf, st + T::ST_F);
    }
    __syncthreads();  // stage s, h and the F16 working copy are free again

    if (STAGES > 1 && tid == 0) {
      const int tn = t + STAGES * stride;
      if (tn < num_tiles) {
        int nx0, ny0;
        tile_origin(tn, nx0, ny0);
        fence_proxy_async_smem();
        issue_tile<T, F16>(st, &bars[s], &tm_b, &tm_d, &tm_f, nx0, ny0, a.drop_loads);
      }
    }
  }
}

// ---- the batched kernel ------------------------------------------------------
// Makes the tensor-map proxy observe the current contents of a tensor map in
// global memory (written by the host since the proxy may last have read that
// address).
__device__ __forceinline__ void tensormap_acquire(const void* tm) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                   reinterpret_cast<uint64_t>(tm))
               : "memory");
}

// Many grids of different sizes advance in one launch.  Work units are the
// tiles of every member grid; CTA u takes units[u], which names its grid and
// tile, so one load stands between the CTA's start and its tile load (the
// single-grid kernel has none).  One CTA per unit (the rest of the launch
// returns at once): a persistent loop over units would keep its state live
// across the tile and push the tile code into register spills.  Launch
// `launch_idx` of a chain skips grids that have taken all their launches, so
// grids with different step counts share a chain.  The CTA then runs the
// same per-tile steps as step_kernel.
template <int K, int TX, int TY, bool F16, bool UNI, int MINB>
__global__ void __launch_bounds__(kThreads, MINB)
    batch_kernel(const BatchGrid* __restrict__ grids, const BatchUnit* __restrict__ units,
                 int launch_idx) {
  using T = Tile<K, TX, TY, F16, 1, UNI>;
  const int4 un = __ldg(reinterpret_cast<const int4*>(units) + blockIdx.x);
  if (launch_idx >= (un.w & 0x3fffffff)) return;
  const BatchGrid& G = grids[un.x];
  const int x0 = un.y, y0 = un.z;
  const int p = ((un.w >> 30) + launch_idx) & 1;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = align_smem(smem_raw);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::OFF_BAR);
  float* sb = reinterpret_cast<float*>(smem + T::ST_B);
  float* sd = reinterpret_cast<float*>(smem + T::ST_D);
  float* sh = T::H_ALIAS ? sb : reinterpret_cast<float*>(smem + T::OFF_H);
  float4* sf = (F16 && !UNI) ? reinterpret_cast<float4*>(smem + T::OFF_WORK)
                             : reinterpret_cast<float4*>(smem + T::ST_F);
  const int tid = threadIdx.x;
  const StepArgs& a = G.a;
  // the unit and grid tables are written before the chain, the state by the
  // previous launch: wait for it before the tile load
  wait_previous_launch();
  allow_next_launch();
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
    const CUtensorMap* tm = G.tm;
    if (G.fence) {
      tensormap_acquire(tm);
      tensormap_acquire(tm + 1 + p);
      tensormap_acquire(tm + 3 + p);
    }
    issue_tile<T, F16>(smem, bar, tm, tm + 1 + p, tm + 3 + p, x0, y0, a.drop_loads);
  }
  uint32_t mask = 0;
#pragma unroll
  for (int k = 0; k < TWS_MAX_SOURCES; ++k) {
    if (k < a.nsrc) {
      const DevSource& src = a.src[k];
      if (src.bx1 >= x0 - T::HX && src.bx0 < x0 + TX + T::HX && src.by1 >= y0 - T::HY &&
          src.by0 < y0 + TY + T::HY)
        mask |= 1u << k;
    }
  }
  __syncthreads();  // the barrier is initialised before anyone waits on it
  const bool ok = wait_bounded(bar, 0, a.err, a.wait_cycles);
  if (__syncthreads_or(!ok)) return;
  const int gw = a.W, gh = a.H;
  const bool interior =
      x0 - T::HX >= 0 && y0 - T::HY >= 0 && x0 + TX + T::HX <= gw && y0 + TY + T::HY <= gh;
  if constexpr (UNI) {
    if (interior)
      process_tile_flat<K, TX, TY, F16, 1, true>(a, G.d[p ^ 1], G.f[p ^ 1], G.v, x0, y0, mask, sb,
                                                 sd, sh, smem + T::ST_F);
    else
      process_tile_flat<K, TX, TY, F16, 1, false>(a, G.d[p ^ 1], G.f[p ^ 1], G.v, x0, y0, mask,
                                                  sb, sd, sh, smem + T::ST_F);
  } else if (interior) {
    process_tile<K, TX, TY, F16, 1, true>(a, G.d[p ^ 1], G.f[p ^ 1], G.v, x0, y0, mask, sb,
                                               sd, sh, sf, smem + T::ST_F);
  } else {
    process_tile<K, TX, TY, F16, 1, false>(a, G.d[p ^ 1], G.f[p ^ 1], G.v, x0, y0, mask, sb,
                                                sd, sh, sf, smem + T::ST_F);
  }
}

// ---- variant table -------------------------------------------------------------
using KernelFn = void (*)(CUtensorMap, CUtensorMap, CUtensorMap, StepArgs);

struct VariantEntry {
  StepVariant v;
  const void* fn[2];  // [flux storage]
  size_t smem[2];
  int ctas_per_sm[2] = {0, 0};  // occupancy, filled on first launch
  bool attr_set[2] = {false, false};
};

template <int K, int TX, int TY, int STAGES, bool UNI>
VariantEntry make_entry() {
  using T32 = Tile<K, TX, TY, false, STAGES, UNI>;
  using T16 = Tile<K, TX, TY, true, STAGES, UNI>;
  VariantEntry e;
  e.v.k = K;
  e.v.tx = TX;
  e.v.ty = TY;
  e.v.stages = STAGES;
  e.v.kind = kKindTile;
  e.v.ry = 0;
  e.v.hx = T32::HX;
  e.v.bw = T32::BW;
  e.v.bh = T32::BH;
  e.v.fw = T32::FW;
  e.v.fh = T32::FH;
  e.v.sw = T32::SW;
  e.v.uni = UNI;
  e.v.smem = T32::SMEM > T16::SMEM ? T32::SMEM : T16::SMEM;
  e.fn[TWS_FLUX_F32] = reinterpret_cast<const void*>(&step_kernel<K, TX, TY, false, STAGES, UNI>);
  e.fn[TWS_FLUX_F16] = reinterpret_cast<const void*>(&step_kernel<K, TX, TY, true, STAGES, UNI>);
  e.smem[TWS_FLUX_F32] = T32::SMEM;
  e.smem[TWS_FLUX_F16] = T16::SMEM;
  return e;
}

struct VariantTable {
  static constexpr int kMax = 48;
  VariantEntry e[kMax + 1];  // one spare slot: an entry past kMax is dropped, not written over n
  int n = 0;
  std::mutex mu;
  VariantTable() {
    // Entries 0..3 are the first tile choice for K = 1..4 in the separate
    // layout (measured on 4096^2: one CTA per tile with a small shared-memory
    // footprint beats persistent double-buffered CTAs, which hold fewer CTAs
    // per SM); step_variant_for names the default per K.
    add<1, 32, 32, 1>();  // 0  plain
    add<2, 64, 16, 1>();  // 1
    add<3, 64, 32, 1>();  // 2
    add<4, 64, 32, 1>();  // 3
    add<1, 64, 16, 1>();  // 4
    add<1, 32, 16, 1>();  // 5
    add<1, 64, 32, 1>();  // 6
    add<1, 16, 32, 1>();  // 7
    add<1, 32, 32, 2>();  // 8  persistent, next tile prefetched
    add<1, 64, 16, 2>();  // 9
    add<2, 32, 32, 1>();  // 10
    add<2, 64, 16, 2>();  // 11
    add<2, 64, 32, 1>();  // 12
    add_stream(64);       // 13 register streaming, 30-column strips x 64 rows
    add_stream(32);       // 14
    add_stream(128);      // 15
    // unified layout: flux box = b/d box, interior tiles walk flat runs
    add<2, 32, 32, 1, true>();  // 16
    add<2, 64, 16, 1, true>();  // 17
    add<3, 32, 32, 1, true>();  // 18
    add<3, 64, 16, 1, true>();  // 19
    add<4, 32, 32, 1, true>();  // 20
    add<4, 64, 16, 1, true>();  // 21
    add<3, 64, 32, 1, true>();  // 22
    // row sweeps: 64-column warp strips, K time levels on chip.  4096^2 FP32
    // (Gcell-steps/s): K = 3 with 32-row bands 211.9, 40 211.6, 48 205.2, 64
    // 184.4; K = 2 171-173; K = 4 173 with 64-row bands.  A ring of 4 rows is
    // 0.3-1.5% faster than 3, one of 8 no faster than 4.
    add_sweep(2, 32, 4);   // 23
    add_sweep(2, 48, 4);   // 24
    add_sweep(3, 32, 4);   // 25
    add_sweep(3, 40, 4);   // 26  the default for large FP32 grids
    add_sweep(3, 48, 4);   // 27
    add_sweep(3, 64, 4);   // 28
    add_sweep(4, 64, 4);   // 29
    // Taller bands, the last ones short (the tail: about one short unit per
    // resident warp ends the work queue).  Tall bands recompute fewer halo
    // rows per output row, and the tail keeps the launch's end short.
    // K = 3 (Gcell-steps/s, FP32 / FP16 flux): 6144^2 80/32 234.5 / 219.4;
    // 8192^2 192/48 253.1 / 237.6; 16384^2 128/48 272.0 / 268.8, 192/48
    // 276.8 / 275.4, 256/64 272.6 / 275.3 (64 rows: 258.8 / 251.4).
    add_sweep(3, 80, 4, 32);   // 30
    add_sweep(3, 128, 4, 48);  // 31
    add_sweep(3, 192, 4, 48);  // 32
    add_sweep(3, 256, 4, 64);  // 33
  }
  void add_sweep(int k, int rows, int ring, int tail_rows = 0) {
    VariantEntry s{};
    s.v.ry_tail = tail_rows;
    s.v.k = k;
    s.v.tx = sweep_valid_columns(k);
    s.v.ty = rows;
    s.v.stages = 1;
    s.v.kind = kKindSweep;
    s.v.ry = rows;
    s.v.ring = ring;
    s.v.smem = sweep_smem_bytes(k, TWS_FLUX_F32, ring);
    e[n] = s;
    if (n < kMax) ++n;
  }
  template <int K, int TX, int TY, int STAGES, bool UNI = false>
  void add() {
    e[n] = make_entry<K, TX, TY, STAGES, UNI>();
    if (n < kMax) ++n;
  }
  void add_stream(int ry) {
    VariantEntry s{};
    s.v.k = 1;
    s.v.tx = 30;
    s.v.ty = ry;
    s.v.stages = 1;
    s.v.kind = kKindStream;
    s.v.ry = ry;
    s.v.smem = 0;
    e[n] = s;
    if (n < kMax) ++n;
  }
};

VariantTable& table() {
  static VariantTable t;
  return t;
}

using EncodeTiledFn = PFN_cuTensorMapEncodeTiled_v12000;

EncodeTiledFn encode_fn(std::string* why) {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    const cudaError_t err =
        cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
    if (err == cudaSuccess && q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  if (!fn && why) *why = "cuTensorMapEncodeTiled is not available from the driver";
  return fn;
}

}  // namespace

int step_variant_count() { return table().n; }
const StepVariant& step_variant(int i) { return table().e[i].v; }

int step_variant_large_grid(int flux_storage, int W, int H) {
  // The three-step row sweep: FP32 flux from kLargeGridCells on (4096^2:
  // 40-row bands, 202.8 Gcell-steps/s against 193.4 for the two-step tiles),
  // FP16 flux from kLargeF16Cells on (6144^2: 219.4 against 209.0 for the
  // FP16 tiles; below it the tiles are as fast or faster: 4096^2 203.7
  // against 184.9).  The band height is the tallest rung of a
  // ladder that leaves at least 2.5 units per resident warp (four CTAs of four
  // warps per SM), measured on 4096^2 to 16384^2.
  const long long cells = (long long)W * H;
  if (cells < kLargeGridCells) return -1;
  if (flux_storage != TWS_FLUX_F32 && cells < kLargeF16Cells) return -1;
  static const int kLadder[][2] = {{40, 0}, {80, 32}, {128, 48}, {192, 48}, {256, 64}};
  static const int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    return cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0
               ? n
               : 1;
  }();
  const double warps = (double)sms * 4 * (kSweepCtaThreads / 32);
  const long long strips = (W + sweep_valid_columns(3) - 1) / sweep_valid_columns(3);
  int pick = -1;
  for (int r = 0; r < (int)(sizeof(kLadder) / sizeof(kLadder[0])); ++r) {
    const long long units = strips * ((H + kLadder[r][0] - 1) / kLadder[r][0]);
    if (r > 0 && units < 2.5 * warps) break;
    for (int i = 0; i < step_variant_count(); ++i) {
      const StepVariant& e = step_variant(i);
      if (e.kind == kKindSweep && e.k == 3 && e.ry == kLadder[r][0] &&
          e.ry_tail == kLadder[r][1])
        pick = i;
    }
  }
  return pick;
}

int step_variant_for(int k, int /*flux_storage*/) {
  // Default variant per temporal depth (fastest per depth on 4096^2): the
  // plain 32x32 kernel for K = 1, the unified-layout 32x32 tiles for K > 1.
  switch (k) {
    case 1: return 0;
    case 2: return 16;
    case 3: return 18;
    case 4: return 20;
    default: return -1;
  }
}

cudaError_t encode_step_maps(int variant, int flux_storage, int W, int H, int pitch,
                             const float* b, const float* d, const void* f, CUtensorMap* tm_b,
                             CUtensorMap* tm_d, CUtensorMap* tm_f, std::string* why) {
  EncodeTiledFn enc = encode_fn(why);
  if (!enc) return cudaErrorNotSupported;
  const StepVariant& v = step_variant(variant);
  const cuuint32_t estr[3] = {1, 1, 1};
  // b and d: 2-D float {W, H}.
  const cuuint64_t gdim2[2] = {(cuuint64_t)W, (cuuint64_t)H};
  const cuuint64_t gstr2[1] = {(cuuint64_t)pitch * 4};
  const cuuint32_t box2[2] = {(cuuint32_t)v.bw, (cuuint32_t)v.bh};
  CUresult r;
  if (b) {
    r = enc(tm_b, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(b), gdim2, gstr2, box2,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      if (why) *why = "tensor map for terrain failed, CUresult " + std::to_string((int)r);
      return cudaErrorInvalidValue;
    }
  }
  if (d) {
    r = enc(tm_d, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(d), gdim2, gstr2, box2,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      if (why) *why = "tensor map for depth failed, CUresult " + std::to_string((int)r);
      return cudaErrorInvalidValue;
    }
  }
  if (f) {
    if (flux_storage == TWS_FLUX_F32) {
      // 3-D float {4 channels, W, H}: one 16-byte record per cell.
      const cuuint64_t gdim[3] = {4, (cuuint64_t)W, (cuuint64_t)H};
      const cuuint64_t gstr[2] = {16, (cuuint64_t)pitch * 16};
      const cuuint32_t box[3] = {4, (cuuint32_t)v.fw, (cuuint32_t)v.fh};
      r = enc(tm_f, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(f), gdim, gstr, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    } else {
      // 3-D half {8 = two cells x 4 channels, ceil(W/2) cell pairs, H}.  The
      // box (the staging width, whole pairs) starts on an even cell; the
      // padding cell of an odd-width row is kept at zero.
      const cuuint64_t gdim[3] = {8, (cuuint64_t)((W + 1) / 2), (cuuint64_t)H};
      const cuuint64_t gstr[2] = {16, (cuuint64_t)pitch * 8};
      const cuuint32_t box[3] = {8, (cuuint32_t)(v.sw / 2), (cuuint32_t)v.fh};
      r = enc(tm_f, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<void*>(f), gdim, gstr, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    }
    if (r != CUDA_SUCCESS) {
      if (why) *why = "tensor map for flux failed, CUresult " + std::to_string((int)r);
      return cudaErrorInvalidValue;
    }
  }
  return cudaSuccess;
}

cudaError_t launch_step(int variant, int flux_storage, const CUtensorMap* tm_b,
                        const CUtensorMap* tm_d, const CUtensorMap* tm_f, const float* b,
                        const float* d, const void* f, const StepArgs& a, cudaStream_t s) {
  VariantTable& t = table();
  if (variant < 0 || variant >= t.n) return cudaErrorInvalidValue;
  const int fs = flux_storage == TWS_FLUX_F16 ? TWS_FLUX_F16 : TWS_FLUX_F32;
  VariantEntry& e = t.e[variant];
  if (e.v.kind == kKindStream) return launch_stream_step(e.v.ry, fs, b, d, f, a, s);
  if (e.v.kind == kKindSweep)
    return launch_sweep_step(e.v.k, e.v.ry, e.v.ry_tail, e.v.ring, fs, b, d, f, a, s);
  if (!tm_b || !tm_d || !tm_f) return cudaErrorInvalidValue;
  const void* fn = e.fn[fs];
  const size_t smem = e.smem[fs];
  int ctas_per_sm;
  {
    std::lock_guard<std::mutex> lk(t.mu);
    if (!e.attr_set[fs]) {
      cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (err != cudaSuccess) return err;
      int n = 0;
      err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kThreads, smem);
      if (err != cudaSuccess) return err;
      e.ctas_per_sm[fs] = n > 0 ? n : 1;
      e.attr_set[fs] = true;
    }
    ctas_per_sm = e.ctas_per_sm[fs];
  }
  const StepVariant& v = e.v;
  const int tiles_x = (a.W + v.tx - 1) / v.tx, tiles_y = (a.H + v.ty - 1) / v.ty;
  dim3 grid(tiles_x, tiles_y);  // one CTA per tile
  if (v.stages > 1) {           // persistent: as many CTAs as fit at once
    static int sms = 0;
    if (sms == 0) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (sms <= 0) sms = 1;
    }
    grid = dim3((unsigned)std::min<long long>((long long)tiles_x * tiles_y,
                                              (long long)sms * ctas_per_sm));
  }
  if (grid.y > 65535) return cudaErrorInvalidConfiguration;
  auto kfn = reinterpret_cast<KernelFn>(const_cast<void*>(fn));
  // programmatic dependent launch: the kernel waits for the previous launch
  // before it touches global memory (wait_previous_launch)
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t launched = cudaLaunchKernelEx(&cfg, kfn, *tm_b, *tm_d, *tm_f, a);
  count_launch();
  return launched;
}

// ---- batched variants ---------------------------------------------------------
namespace {

using BatchFn = void (*)(const BatchGrid*, const BatchUnit*, int);

struct BatchEntry {
  int k, tx, ty, uni;
  int step_variant;  // the single-grid variant with the same boxes (its tensor maps fit)
  const void* fn[2];
  size_t smem[2];
  int ctas_per_sm[2] = {0, 0};
  bool set[2] = {false, false};
};

// MINB: CTAs per SM the register allocation must allow (the batched kernel
// keeps its grid's scalars in registers, where the single-grid kernel reads
// them from the parameter bank).
template <int K, int TX, int TY, bool UNI, int MINB>
BatchEntry make_batch_entry(int step_variant) {
  BatchEntry e;
  e.k = K;
  e.tx = TX;
  e.ty = TY;
  e.uni = UNI;
  e.step_variant = step_variant;
  e.fn[TWS_FLUX_F32] = reinterpret_cast<const void*>(&batch_kernel<K, TX, TY, false, UNI, MINB>);
  e.fn[TWS_FLUX_F16] = reinterpret_cast<const void*>(&batch_kernel<K, TX, TY, true, UNI, MINB>);
  e.smem[TWS_FLUX_F32] = Tile<K, TX, TY, false, 1, UNI>::SMEM;
  e.smem[TWS_FLUX_F16] = Tile<K, TX, TY, true, 1, UNI>::SMEM;
  return e;
}

struct BatchTable {
  BatchEntry e[8];
  int n = 0;
  std::mutex mu;
  BatchTable() {
    e[n++] = make_batch_entry<1, 32, 32, false, 5>(0);
    e[n++] = make_batch_entry<2, 32, 32, false, 5>(10);
    e[n++] = make_batch_entry<1, 64, 16, false, 5>(4);
    e[n++] = make_batch_entry<2, 64, 16, false, 5>(1);
    e[n++] = make_batch_entry<2, 32, 32, true, 5>(16);
    e[n++] = make_batch_entry<2, 64, 16, true, 5>(17);
    e[n++] = make_batch_entry<3, 32, 32, true, 3>(18);
  }
};

BatchTable& batch_table() {
  static BatchTable t;
  return t;
}

}  // namespace

int batch_variant_count() { return batch_table().n; }
int batch_variant_default() { return 4; }

void batch_variant_info(int i, int* k, int* tx, int* ty, int* step_variant) {
  const BatchEntry& e = batch_table().e[i];
  if (k) *k = e.k;
  if (tx) *tx = e.tx;
  if (ty) *ty = e.ty;
  if (step_variant) *step_variant = e.step_variant;
}

cudaError_t prepare_batch_variant(int variant, int flux_storage) {
  BatchTable& t = batch_table();
  if (variant < 0 || variant >= t.n) return cudaErrorInvalidValue;
  const int fs = flux_storage == TWS_FLUX_F16 ? TWS_FLUX_F16 : TWS_FLUX_F32;
  BatchEntry& e = t.e[variant];
  const StepVariant& sv = step_variant(e.step_variant);
  if (sv.k != e.k || sv.tx != e.tx || sv.ty != e.ty || sv.uni != e.uni || sv.stages != 1)
    return cudaErrorInvalidValue;  // the tables disagree: the maps would not fit
  std::lock_guard<std::mutex> lk(t.mu);
  if (!e.set[fs]) {
    cudaError_t err =
        cudaFuncSetAttribute(e.fn[fs], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e.smem[fs]);
    if (err != cudaSuccess) return err;
    int n = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, e.fn[fs], kThreads, e.smem[fs]);
    if (err != cudaSuccess) return err;
    e.ctas_per_sm[fs] = n > 0 ? n : 1;
    e.set[fs] = true;
  }
  return cudaSuccess;
}

cudaError_t launch_batch_step(int variant, int flux_storage, const BatchGrid* grids,
                              const BatchUnit* units, int launch_idx, int blocks,
                              cudaStream_t s) {
  cudaError_t err = prepare_batch_variant(variant, flux_storage);
  if (err != cudaSuccess) return err;
  if (blocks <= 0) return cudaErrorInvalidValue;
  const int fs = flux_storage == TWS_FLUX_F16 ? TWS_FLUX_F16 : TWS_FLUX_F32;
  BatchEntry& e = batch_table().e[variant];
  auto fn = reinterpret_cast<BatchFn>(const_cast<void*>(e.fn[fs]));
  // programmatic dependent launch, as for the single-grid step kernels
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)blocks, 1, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = e.smem[fs];
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t launched = cudaLaunchKernelEx(&cfg, fn, grids, units, launch_idx);
  count_launch();
  return launched;
}

}  // namespace tws
