// tws_sweep.cu -- the temporally blocked step as a row sweep.
//
// Same arithmetic as the tiled kernels (flowUpdate.comp:34-62 then
// flowApply.comp:32-52, K steps per launch, bit-identical to the FP32
// transcription of the shaders), organised so that no halo is recomputed in y:
//
// * A warp owns a strip of 64 columns (two per lane) and sweeps it down a
//   band of R rows; the warps are persistent and take (strip, band) units
//   from a per-grid queue, border units first, short bands last.  Each lane
//   keeps, per time level s = 0..K-1, a rolling window of the rows that level
//   needs: surface heights h of three rows, depths and terrain of two rows in
//   registers, the new outflows of two rows in shared memory (the registers
//   they would take cost a CTA per SM).
//   Row by row, level s computes the outflow of one row and the depth of the
//   row above, which is the input row of level s + 1 two rows further up; the
//   last level writes its depth, flux and flow map.  The y neighbours come
//   from the window, the x neighbours from the lane itself or its neighbour
//   lanes (warp shuffles).  Values of the two outermost columns of the strip
//   go stale one more column per phase, so a strip yields 64 - 4K output
//   columns; neighbouring strips overlap by 4K columns (their loads are L2
//   hits).  A band also loads 2K rows above and below it, whose results are
//   not written.
// * The two columns of a lane are one packed f32x2 operand
//   (add/sub/mul.rn.f32x2): each lane of it is the IEEE round-to-nearest
//   result of its own operands.  A packed product never feeds a packed sum
//   (the assembler would contract the pair into a fused multiply-add); those
//   sums are scalar.
// * Loads: each lane copies its own two cells of a row (b, d, the flux
//   records) into a private ring of P rows in shared memory with cp.async,
//   P - 1 rows ahead of the row it computes.  Cells off the grid are
//   zero-filled by the copy itself (the shaders' out-of-range image loads
//   read zero).  A lane reads back only what it copied, so no barrier is
//   needed; cp.async.wait_group is the hardware's wait, and a slot is
//   refilled only in the iteration after the one that read it into
//   registers and used those values.
//
// HBM traffic per launch: the state once in, once out (52 B per cell for FP32
// flux, 36 B for FP16), plus the re-read of the strip and band overlaps,
// which L2 serves when neighbouring strips run together.

#include <algorithm>
#include <map>
#include <mutex>

#include "tws_device.cuh"
#include "tws_internal.h"

namespace tws {
namespace {

constexpr int kSweepThreads = kSweepCtaThreads;
constexpr int kSweepWarps = kSweepThreads / 32;
constexpr int kSweepCols = 64;  // columns a warp loads

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// cp.async of `bytes` (<= size) from src; the rest of the `size` bytes is zero.
__device__ __forceinline__ void copy8(void* dst, const void* src, int bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_addr(dst)), "l"(src),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void copy16(void* dst, const void* src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(src),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void copy_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void copy_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// The four outflow channels (+x, -x, +y, -y) of a lane's two cells: .x of
// each float2 is the lane's first column, .y its second.
struct Flux2 {
  float2 x, y, z, w;
};
__device__ __forceinline__ Flux2 zero_flux() {
  const float2 z = make_float2(0.0f, 0.0f);
  return Flux2{z, z, z, z};
}

__device__ __forceinline__ float2 max0x2(float2 v) {
  return make_float2(max0_fast(v.x), max0_fast(v.y));
}
// p + q per column, with p and q packed products: scalar sums (never fadd2
// of an fmul2 result, see the file comment)
__device__ __forceinline__ float2 sum_products(float2 p, float2 q) {
  return make_float2(fadd(p.x, q.x), fadd(p.y, q.y));
}

// Shared memory of one warp, in bytes.
constexpr int sweep_row_bytes(bool f16) { return 512 + (f16 ? 512 : 1024); }
constexpr int kSweepSlotBytes = 1024;
constexpr int sweep_warp_bytes(int k, bool f16, int ring) {
  return sweep_row_bytes(f16) * ring + k * 2 * kSweepSlotBytes;
}

template <int K, bool F16, int P>
struct SweepRing {
  // one row of a lane's ring: b and d of its two cells, then the flux records
  // (FP32: the first cells of all lanes, then the second cells, so that a
  // warp's 16-byte reads are conflict-free; FP16: both cells' 8 halves)
  static constexpr int B = 0;    // 64 floats
  static constexpr int D = 256;  // 64 floats
  static constexpr int F = 512;  // FP32: 2 x 32 float4; FP16: 32 x 16 bytes
  static constexpr int ROW = sweep_row_bytes(F16);
  static constexpr int RING = ROW * P;  // P rows: P - 1 in flight
  // The new outflows of each level's two previous rows, one 1 KB slot per
  // row (the row computed in an iteration takes the slot of the older one
  // once it has been read): each lane's (+x, -x) pairs at 16 * lane, its
  // (+y, -y) pairs at 512 + 16 * lane.
  static constexpr int NSLOT = kSweepSlotBytes;
  static constexpr int WARP = sweep_warp_bytes(K, F16, P);
};

template <int K, bool F16, bool INTERIOR, int P>
__device__ __forceinline__ void sweep_unit(const StepArgs& a, const float* __restrict__ gb,
                                           const float* __restrict__ gd,
                                           const void* __restrict__ gf,
                                           float* __restrict__ d_out, void* __restrict__ f_out,
                                           float2* __restrict__ v_out, unsigned char* ring,
                                           int xs, int y0, int R, uint32_t mask) {
  using RG = SweepRing<K, F16, P>;
  constexpr int HALO = 2 * K;
  const int lane = threadIdx.x & 31;
  const int W = a.W, H = a.H;
  const size_t pitch = (size_t)a.pitch;
  const float2 kf2 = make_float2(a.kf, a.kf), ka2 = make_float2(a.ka, a.ka);
  const float2 cc2 = make_float2(a.c, a.c);
  const float fscale = a.flux_scale, finv = a.flux_inv_scale;
  const float2 fscale2 = make_float2(fscale, fscale), finv2 = make_float2(finv, finv);
  const bool closed = a.closed != 0;

  // this lane's columns
  const int gx0 = xs + 2 * lane, gx1 = gx0 + 1;
  const bool in0 = INTERIOR || (gx0 >= 0 && gx0 < W);
  const bool in1 = INTERIOR || (gx1 >= 0 && gx1 < W);
  const bool out_lane = lane >= K && lane < 32 - K;  // columns HALO .. 63 - HALO
  const int first_row = y0 - HALO;
  const int rows = R + 2 * HALO;  // rows loaded

  // ---- the copies of row r into ring slot `slot`
  auto issue_row = [&](int r, int slot) {
    unsigned char* st = ring + slot * RG::ROW;
    const bool row_in = INTERIOR || (r >= 0 && r < H);
    const int nb = (row_in && in0) ? (in1 ? 8 : 4) : 0;
    const size_t g = row_in ? (size_t)r * pitch + (size_t)(in0 ? gx0 : 0) : 0;
    copy8(st + RG::B + 8 * lane, gb + g, nb);
    copy8(st + RG::D + 8 * lane, gd + g, nb);
    if constexpr (F16) {
      copy16(st + RG::F + 16 * lane, reinterpret_cast<const uint2*>(gf) + g, nb * 2);
    } else {
      const float4* f4 = reinterpret_cast<const float4*>(gf);
      copy16(st + RG::F + 16 * lane, f4 + g, (row_in && in0) ? 16 : 0);
      copy16(st + RG::F + 512 + 16 * lane, f4 + g + ((row_in && in1) ? 1 : 0),
             (row_in && in1) ? 16 : 0);
    }
  };
  auto read_bd = [&](int slot, float2& b, float2& d) {
    const unsigned char* st = ring + slot * RG::ROW;
    b = *reinterpret_cast<const float2*>(st + RG::B + 8 * lane);
    d = *reinterpret_cast<const float2*>(st + RG::D + 8 * lane);
  };
  auto read_flux = [&](int slot) -> Flux2 {
    const unsigned char* st = ring + slot * RG::ROW;
    if constexpr (F16) {
      const uint4 raw = *reinterpret_cast<const uint4*>(st + RG::F + 16 * lane);
      const float2 a0 = fmul2(__half22float2(*reinterpret_cast<const __half2*>(&raw.x)), finv2);
      const float2 a1 = fmul2(__half22float2(*reinterpret_cast<const __half2*>(&raw.y)), finv2);
      const float2 b0 = fmul2(__half22float2(*reinterpret_cast<const __half2*>(&raw.z)), finv2);
      const float2 b1 = fmul2(__half22float2(*reinterpret_cast<const __half2*>(&raw.w)), finv2);
      return Flux2{make_float2(a0.x, b0.x), make_float2(a0.y, b0.y), make_float2(a1.x, b1.x),
                   make_float2(a1.y, b1.y)};
    } else {
      const float4 c0 = *reinterpret_cast<const float4*>(st + RG::F + 16 * lane);
      const float4 c1 = *reinterpret_cast<const float4*>(st + RG::F + 512 + 16 * lane);
      return Flux2{make_float2(c0.x, c1.x), make_float2(c0.y, c1.y), make_float2(c0.z, c1.z),
                   make_float2(c0.w, c1.w)};
    }
  };
  // The sources of row r on this lane's two cells, in source order (as
  // add_sources applies them).  A DISK is tested inline: an out-of-line call
  // per cell and level made the warps under a rain disk several times slower
  // than the rest, and with one wave of warps the launch waits for them.
  auto sources2 = [&](float2 dv, int r) -> float2 {
    if (!mask || !(INTERIOR || (r >= 0 && r < H))) return dv;
#pragma unroll 1
    for (int k = 0; k < a.nsrc; ++k) {
      if (!((mask >> k) & 1u)) continue;
      const DevSource& src = a.src[k];
      if (r < src.by0 || r > src.by1) continue;  // warp-uniform
      if (src.kind == TWS_SOURCE_DISK) {
        const long long dy = r - src.icy;
        const long long room = (long long)src.ir * src.ir - dy * dy;  // dx^2 allowed
        const long long dx0 = gx0 - src.icx, dx1 = gx1 - src.icx;
        if (in0 && gx0 >= src.bx0 && gx0 <= src.bx1 && dx0 * dx0 <= room)
          dv.x = add_rain(dv.x, src.rate, gx0, r);
        if (in1 && gx1 >= src.bx0 && gx1 <= src.bx1 && dx1 * dx1 <= room)
          dv.y = add_rain(dv.y, src.rate, gx1, r);
      } else {
        if (in0) dv.x = add_sources(dv.x, gx0, r, a, 1u << k);
        if (in1) dv.y = add_sources(dv.y, gx1, r, a, 1u << k);
      }
    }
    return dv;
  };

  // ---- per-level windows (registers; every index below is a compile-time
  // constant once the level loops are unrolled)
  float2 H0[K], H1[K];  // h of rows ys - 1 and ys of level s's outflow row ys
  float2 D0[K], D1[K];  // d of rows ys - 1 and ys
  float2 B0[K], B1[K];  // terrain of rows ys - 1 and ys (it travels with the rows)
  // The new outflows of rows ys - 1 and ys - 2 live in shared memory (two
  // slots per level, swapped every iteration), which leaves registers for
  // four CTAs per SM.  A lane reads back only what it wrote.
  unsigned char* const nring = ring + RG::RING;
  auto n_slot = [&](int s, int q) { return nring + (s * 2 + q) * RG::NSLOT; };
  auto store_n = [&](int s, int q, const Flux2& v) {
    unsigned char* sl = n_slot(s, q);
    *reinterpret_cast<float4*>(sl + 16 * lane) = make_float4(v.x.x, v.x.y, v.y.x, v.y.y);
    *reinterpret_cast<float4*>(sl + 512 + 16 * lane) = make_float4(v.z.x, v.z.y, v.w.x, v.w.y);
  };
  auto load_n = [&](int s, int q) -> Flux2 {
    const unsigned char* sl = n_slot(s, q);
    const float4 p = *reinterpret_cast<const float4*>(sl + 16 * lane);
    const float4 m = *reinterpret_cast<const float4*>(sl + 512 + 16 * lane);
    return Flux2{make_float2(p.x, p.y), make_float2(p.z, p.w), make_float2(m.x, m.y),
                 make_float2(m.z, m.w)};
  };
  auto load_n_z = [&](int s, int q) -> float2 {  // the +y pair alone
    return *reinterpret_cast<const float2*>(n_slot(s, q) + 512 + 16 * lane);
  };
  const float2 z2 = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int s = 0; s < K; ++s) {
    H0[s] = H1[s] = D0[s] = D1[s] = B0[s] = B1[s] = z2;
    for (int q = 0; q < 2; ++q) store_n(s, q, zero_flux());
  }
  int q_prev = 1, q_prev2 = 0;  // slots of rows ys - 1 and ys - 2

  // the ring: rows 0 .. P - 2 in flight before the loop
#pragma unroll
  for (int i = 0; i < P - 1; ++i) {
    if (i < rows) issue_row(first_row + i, i);
    copy_commit();
  }
  Flux2 fin_prev = zero_flux();  // flux of the previously loaded row

  // FP16 storage: two rows per loop trip (the windows shift by register
  // renaming; 16384^2 264 -> 272 Gcell-steps/s); FP32 gains nothing from it
#pragma unroll(F16 ? 2 : 1)
  for (int t = 0; t < rows; ++t) {
    const int r = first_row + t;
    const int slot = t % P;
    // refill the slot of row r - 1 (read in full in the previous iteration)
    // with row r + P - 1, then wait for row r
    if (t + P - 1 < rows) issue_row(first_row + t + P - 1, (t + P - 1) % P);
    copy_commit();
    copy_wait<P - 1>();
    float2 bl, dl;
    read_bd(slot, bl, dl);
    const Flux2 fl = read_flux(slot);
    // level 0's input row: the first step's sources, then h = d + b
    float2 d_in = sources2(dl, r);
    float2 h_in = fadd2(d_in, bl);
    float2 b_in = bl;
    Flux2 f_in = fin_prev;  // flux of row r - 1: level 0's outflow row
    fin_prev = fl;

#pragma unroll
    for (int s = 0; s < K; ++s) {
      const int ys = r - 2 * s - 1;  // this level's outflow row
      const bool ys_in = INTERIOR || (ys >= 0 && ys < H);
      // this level's outflow rows ys - 1 and ys - 2 from shared memory, read
      // ahead of the arithmetic that hides their latency (row ys - 2's slot
      // is rewritten only after this read, by the same lane)
      const Flux2 own = load_n(s, q_prev);
      Flux2 handoff;  // new outflow of row ys - 2: level s + 1's input
      float2 Y0;
      if (s + 1 < K) {
        handoff = load_n(s, q_prev2);
        Y0 = handoff.z;
      } else {
        Y0 = load_n_z(s, q_prev2);
      }
      // the parts of the depth update that do not need this row's outflow
      // (flowApply.comp:32-39): the x inflows and the outflow sum of row
      // ys - 1, ahead of the outflow's divergent scaling branch
      const float2 X1 = make_float2(own.y.y, __shfl_down_sync(0xffffffffu, own.y.x, 1));
      const float2 X0 = make_float2(__shfl_up_sync(0xffffffffu, own.x.y, 1), own.x.x);
      const float2 in_x = fadd2(X1, X0);
      const float2 out = fadd2(fadd2(fadd2(own.x, own.y), own.z), own.w);

      // -- outflow of row ys, flowUpdate.comp:34-62
      const float2 hm = H0[s], hc = H1[s], hp = h_in;
      const float2 h_right = make_float2(hc.y, __shfl_down_sync(0xffffffffu, hc.x, 1));
      const float2 h_left = make_float2(__shfl_up_sync(0xffffffffu, hc.y, 1), hc.x);
      Flux2 nf;
      {
        const float2 e_px = fsub2(hc, h_right), e_mx = fsub2(hc, h_left);
        const float2 e_py = fsub2(hc, hp), e_my = fsub2(hc, hm);
        nf.x = max0x2(sum_products(fmul2(f_in.x, kf2), fmul2(e_px, ka2)));
        nf.y = max0x2(sum_products(fmul2(f_in.y, kf2), fmul2(e_mx, ka2)));
        nf.z = max0x2(sum_products(fmul2(f_in.z, kf2), fmul2(e_py, ka2)));
        nf.w = max0x2(sum_products(fmul2(f_in.w, kf2), fmul2(e_my, ka2)));
      }
      if constexpr (!INTERIOR) {
        if (closed) {  // no outflow across a closed wall
          if (gx0 + 1 >= W) nf.x.x = 0.0f;
          if (gx1 + 1 >= W) nf.x.y = 0.0f;
          if (gx0 == 0) nf.y.x = 0.0f;
          if (gx1 == 0) nf.y.y = 0.0f;
          if (ys + 1 >= H) nf.z = z2;
          if (ys == 0) nf.w = z2;
        }
      }
      {
        const float2 dc = D1[s];
        const float2 total = fmul2(fadd2(fadd2(fadd2(nf.x, nf.y), nf.z), nf.w), cc2);
        if (total.x > dc.x) {
          const float sc = scale_factor(dc.x, total.x);
          nf.x.x = fmul(nf.x.x, sc);
          nf.y.x = fmul(nf.y.x, sc);
          nf.z.x = fmul(nf.z.x, sc);
          nf.w.x = fmul(nf.w.x, sc);
        }
        if (total.y > dc.y) {
          const float sc = scale_factor(dc.y, total.y);
          nf.x.y = fmul(nf.x.y, sc);
          nf.y.y = fmul(nf.y.y, sc);
          nf.z.y = fmul(nf.z.y, sc);
          nf.w.y = fmul(nf.w.y, sc);
        }
      }
      if constexpr (F16) {
        nf.x = quantize_f16x2(nf.x, fscale2, finv2);
        nf.y = quantize_f16x2(nf.y, fscale2, finv2);
        nf.z = quantize_f16x2(nf.z, fscale2, finv2);
        nf.w = quantize_f16x2(nf.w, fscale2, finv2);
      }
      if constexpr (!INTERIOR) {  // cells off the grid keep zero outflow
        if (!ys_in) nf = zero_flux();
        if (!in0) nf.x.x = nf.y.x = nf.z.x = nf.w.x = 0.0f;
        if (!in1) nf.x.y = nf.y.y = nf.z.y = nf.w.y = 0.0f;
      }

      store_n(s, q_prev2, nf);  // row ys takes the slot of ys - 2, read above

      // -- depth and flow map of row ys - 1, flowApply.comp:32-52
      const int yd = ys - 1;
      const float2 Y1 = nf.w;
      const float2 in = fadd2(fadd2(in_x, Y1), Y0);
      const float2 dn = max0x2(sum_products(D0[s], fmul2(fsub2(in, out), cc2)));
      const float2 b_d = B0[s];  // terrain of the depth row
      // shift the windows
      H0[s] = hc;
      H1[s] = hp;
      D0[s] = D1[s];
      D1[s] = d_in;
      B0[s] = B1[s];
      B1[s] = b_in;
      if (s + 1 < K) {
        // level s + 1's input row yd: next step's sources, h = d + b
        const bool yd_in = INTERIOR || (yd >= 0 && yd < H);
        float2 dnext = dn;
        if constexpr (!INTERIOR) {
          if (!yd_in) dnext = z2;
          if (!in0) dnext.x = 0.0f;
          if (!in1) dnext.y = 0.0f;
        }
        dnext = sources2(dnext, yd);
        d_in = dnext;
        h_in = fadd2(dnext, b_d);
        b_in = b_d;
        f_in = handoff;
      } else if (yd >= y0 && yd < y0 + R && out_lane && (INTERIOR || yd < H)) {
        // the last level: depth, flux and flow map of row yd go out
        const size_t g = (size_t)yd * pitch + (size_t)gx0;
        const float2 vx = fsub2(fsub2(X1, own.x), fsub2(X0, own.y));
        const float2 vy = fsub2(fsub2(Y1, own.z), fsub2(Y0, own.w));
        if (INTERIOR || in1) {
          *reinterpret_cast<float2*>(d_out + g) = dn;
          *reinterpret_cast<float4*>(v_out + g) = make_float4(vx.x, vy.x, vx.y, vy.y);
          if constexpr (F16) {
            const __half2 p0 = __float22half2_rn(fmul2(make_float2(own.x.x, own.y.x), fscale2));
            const __half2 q0 = __float22half2_rn(fmul2(make_float2(own.z.x, own.w.x), fscale2));
            const __half2 p1 = __float22half2_rn(fmul2(make_float2(own.x.y, own.y.y), fscale2));
            const __half2 q1 = __float22half2_rn(fmul2(make_float2(own.z.y, own.w.y), fscale2));
            uint4 packed;
            packed.x = *reinterpret_cast<const uint32_t*>(&p0);
            packed.y = *reinterpret_cast<const uint32_t*>(&q0);
            packed.z = *reinterpret_cast<const uint32_t*>(&p1);
            packed.w = *reinterpret_cast<const uint32_t*>(&q1);
            *reinterpret_cast<uint4*>(reinterpret_cast<uint2*>(f_out) + g) = packed;
          } else {
            float4* fo = reinterpret_cast<float4*>(f_out) + g;
            fo[0] = make_float4(own.x.x, own.y.x, own.z.x, own.w.x);
            fo[1] = make_float4(own.x.y, own.y.y, own.z.y, own.w.y);
          }
        } else if (in0) {  // the grid's last column (odd width)
          d_out[g] = dn.x;
          v_out[g] = make_float2(vx.x, vy.x);
          if constexpr (F16) {
            const __half2 p0 = __float22half2_rn(fmul2(make_float2(own.x.x, own.y.x), fscale2));
            const __half2 q0 = __float22half2_rn(fmul2(make_float2(own.z.x, own.w.x), fscale2));
            uint2 packed;
            packed.x = *reinterpret_cast<const uint32_t*>(&p0);
            packed.y = *reinterpret_cast<const uint32_t*>(&q0);
            reinterpret_cast<uint2*>(f_out)[g] = packed;
          } else {
            reinterpret_cast<float4*>(f_out)[g] =
                make_float4(own.x.x, own.y.x, own.z.x, own.w.x);
          }
        }
      }
    }
    // the row of this iteration becomes ys - 1, its predecessor ys - 2
    const int q_row = q_prev2;
    q_prev2 = q_prev;
    q_prev = q_row;
  }
  copy_wait<0>();
}

// Queue position i -> (strip, band): the units on the grid's border first
// (their cells take the slower edge path, and a launch ends with its slowest
// units), then the interior strip by strip, band by band.
__device__ __forceinline__ void sweep_unit_coords(int i, int S, int B, int& s, int& b) {
  if (S < 3 || B < 3) {
    s = i % S;
    b = i / S;
    return;
  }
  const int ne = 2 * S + 2 * (B - 2);
  if (i < S) {
    s = i;
    b = 0;
  } else if (i < 2 * S) {
    s = i - S;
    b = B - 1;
  } else if (i < 2 * S + (B - 2)) {
    s = 0;
    b = 1 + (i - 2 * S);
  } else if (i < ne) {
    s = S - 1;
    b = 1 + (i - 2 * S - (B - 2));
  } else {
    const int j = i - ne;
    s = 1 + j % (S - 2);
    b = 1 + j / (S - 2);
  }
}

// The bands of a launch: rows [0, tall_end) in bands of `tall` rows (the
// last one may be shorter), then rows [tall_end, H) in bands of `tail` rows.
// Short bands come last in the work queue, so that the launch ends on small
// units; tall bands recompute fewer halo rows per output row.
struct SweepBands {
  int tall, tall_end, tall_count, tail, count;
};

// Band i of a partition with a tail: its first row and its height.
__device__ __forceinline__ void sweep_band(const SweepBands& sb, int H, int i, int& y0, int& R) {
  const bool tall = i < sb.tall_count;
  y0 = tall ? i * sb.tall : sb.tall_end + (i - sb.tall_count) * sb.tail;
  R = min(tall ? sb.tall : sb.tail, (tall ? sb.tall_end : H) - y0);
}

// Persistent warps (one wave): each takes units (strip, band) from the grid's
// queue until none is left, so warps that drew cheap units take more of them.
template <int K, bool F16, int P, bool TAIL>
__global__ void __launch_bounds__(kSweepThreads, (K <= 3 ? 4 : 2))
    sweep_kernel(const float* __restrict__ b, const float* __restrict__ d,
                 const void* __restrict__ f, const __grid_constant__ StepArgs a,
                 const SweepBands sb) {
  using RG = SweepRing<K, F16, P>;
  constexpr int VALID = kSweepCols - 4 * K;
  extern __shared__ __align__(128) unsigned char sweep_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int strips = (a.W + VALID - 1) / VALID;
  const int bands = sb.count;
  const int total = strips * bands;
  // the previous launch on the stream has completed and its writes (the
  // state, and the queue it reset) are visible before any global access
  // (programmatic dependent launch)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  unsigned char* ring = sweep_smem + warp * RG::WARP;
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(&a.queue[0], 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= total) break;  // the whole warp
    int si, bi;
    sweep_unit_coords(u, strips, bands, si, bi);
    const int xs = si * VALID - 2 * K;
    int y0, R;
    if constexpr (TAIL) {
      sweep_band(sb, a.H, bi, y0, R);
    } else {  // uniform bands: the height stays a kernel parameter
      y0 = bi * sb.tall;
      R = sb.tall;
    }
    uint32_t mask = 0;
#pragma unroll
    for (int k = 0; k < TWS_MAX_SOURCES; ++k) {
      if (k < a.nsrc) {
        const DevSource& s = a.src[k];
        if (s.bx1 >= xs && s.bx0 < xs + kSweepCols && s.by1 >= y0 - 2 * K &&
            s.by0 < y0 + R + 2 * K)
          mask |= 1u << k;
      }
    }
    const bool interior =
        xs >= 0 && xs + kSweepCols <= a.W && y0 - 2 * K >= 0 && y0 + R + 2 * K <= a.H;
    if (interior)
      sweep_unit<K, F16, true, P>(a, b, d, f, a.d_out, a.f_out, a.v_out, ring, xs, y0, R, mask);
    else
      sweep_unit<K, F16, false, P>(a, b, d, f, a.d_out, a.f_out, a.v_out, ring, xs, y0, R, mask);
  }
  // The last warp to finish resets the queue for the next launch: every other
  // warp has made its final claim by then, and the next launch reads the
  // queue only after this grid has completed.
  if (lane == 0) {
    __threadfence();
    if (atomicAdd(&a.queue[1], 1) == (int)(gridDim.x * kSweepWarps) - 1) {
      a.queue[0] = 0;
      a.queue[1] = 0;
      __threadfence();
    }
  }
}

template <int K, int P>
const void* sweep_fn(int flux_storage, bool tail) {
  if (flux_storage == TWS_FLUX_F16)
    return tail ? reinterpret_cast<const void*>(&sweep_kernel<K, true, P, true>)
                : reinterpret_cast<const void*>(&sweep_kernel<K, true, P, false>);
  return tail ? reinterpret_cast<const void*>(&sweep_kernel<K, false, P, true>)
              : reinterpret_cast<const void*>(&sweep_kernel<K, false, P, false>);
}

}  // namespace

int sweep_valid_columns(int k) { return kSweepCols - 4 * k; }

size_t sweep_smem_bytes(int k, int flux_storage, int ring) {
  return (size_t)kSweepWarps * sweep_warp_bytes(k, flux_storage == TWS_FLUX_F16, ring);
}

cudaError_t launch_sweep_step(int k, int rows, int tail_rows, int ring, int flux_storage,
                              const float* b, const float* d, const void* f, const StepArgs& a,
                              cudaStream_t s) {
  const void* fn = nullptr;
  if (ring != 4) return cudaErrorInvalidValue;
  switch (k) {
    case 2: fn = sweep_fn<2, 4>(flux_storage, tail_rows > 0); break;
    case 3: fn = sweep_fn<3, 4>(flux_storage, tail_rows > 0); break;
    case 4: fn = sweep_fn<4, 4>(flux_storage, tail_rows > 0); break;
    default: return cudaErrorInvalidValue;
  }
  if (rows < 1 || tail_rows < 0 || !a.queue) return cudaErrorInvalidValue;
  const size_t smem = sweep_smem_bytes(k, flux_storage, ring);
  // one wave of persistent CTAs (occupancy of this instantiation, queried once)
  static std::mutex mu;
  static std::map<const void*, int> resident;
  int per_sm = 0, sms = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = resident.find(fn);
    if (it == resident.end()) {
      cudaError_t e = cudaSuccess;
      if (smem > 48 * 1024)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      int n = 0;
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kSweepThreads, smem);
      if (e != cudaSuccess) return e;
      it = resident.emplace(fn, n > 0 ? n : 1).first;
    }
    per_sm = it->second;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    sms = 1;
  const int valid = kSweepCols - 4 * k;
  const long long strips = (a.W + valid - 1) / valid;
  // Band partition: with a tail, about one short unit per resident warp ends
  // the queue (at most half of the rows).
  SweepBands sb{};
  sb.tall = rows;
  sb.tail = tail_rows > 0 ? tail_rows : rows;
  long long tail_bands = 0;
  if (tail_rows > 0) {
    const long long warps = (long long)per_sm * sms * kSweepWarps;
    tail_bands = std::min<long long>((warps + strips - 1) / strips, a.H / (2LL * tail_rows));
  }
  sb.tall_end = a.H - (int)(tail_bands * sb.tail);
  sb.tall_count = (sb.tall_end + rows - 1) / rows;
  sb.count = sb.tall_count + (int)tail_bands;
  const long long units = strips * sb.count;
  if (units > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const long long blocks =
      std::min<long long>((units + kSweepWarps - 1) / kSweepWarps, (long long)per_sm * sms);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(kSweepThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  using Fn = void (*)(const float*, const float*, const void*, StepArgs, SweepBands);
  const cudaError_t e =
      cudaLaunchKernelEx(&cfg, reinterpret_cast<Fn>(const_cast<void*>(fn)), b, d, f, a, sb);
  count_launch();
  return e;
}

}  // namespace tws
