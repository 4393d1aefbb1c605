// tws_resident.cu -- small grids advanced with their whole state on chip.
//
// One thread-block cluster of 1 to 16 CTAs (one per SM, 1024 threads each)
// holds the grid: CTA `rank` owns rows [rank*R, rank*R + R) in seven planes
// of its shared memory (terrain b, depth d, surface h = d + b, and the four
// outflow channels +x, -x, +y, -y), 28 bytes per cell.  One launch runs many
// steps without touching global memory between them:
//
//   load b, d, f; first step's sources; h = d + b          barrier
//   per step:  outflow (flowUpdate.comp:34-62)               barrier
//              depth + flow map (flowApply.comp:32-52);
//              next step's sources; h = d + b                barrier
//   the last step writes d, f and the flow map to global memory.
//
// The only neighbours outside a CTA's own rows are the row above and the row
// below: the surface height (outflow phase) and the +y / -y outflow (depth
// phase) of the adjacent CTAs' edge rows.  Each CTA keeps ghost rows for them
// in its own planes, and the CTA that computes an edge row writes it into
// its neighbour's ghost row through distributed shared memory, so that both
// phases read plain shared memory only.  Ghost rows beyond the grid stay zero
// (the reference's out-of-range imageLoad).  The cluster barrier (release /
// acquire at cluster scope) orders every phase's shared-memory writes, local
// and remote, before the next phase's reads, and the last barrier keeps each
// CTA alive until no neighbour writes into it any more.  Every thread of every
// CTA executes the same sequence of barriers.  A one-CTA cluster uses block
// barriers only.
//
// The arithmetic is the one of the tiled kernels and the oracle, operation
// for operation (explicit round-to-nearest intrinsics), so results are
// bit-identical to them.

#include <climits>

#include <cooperative_groups.h>

#include "tws_device.cuh"
#include "tws_internal.h"

namespace cg = cooperative_groups;

namespace tws {
namespace {

constexpr int kResThreads = 1024;

// Planes per CTA, in floats, for R rows of width W: b, d (R rows); h with a
// ghost row above and below (R + 2); +x, -x (R); +y with a ghost row above
// (R + 1); -y with a ghost row below (R + 1).
__host__ __device__ constexpr size_t res_floats(int R, int W) {
  return (size_t)(7 * R + 4) * W;
}

struct ResPlanes {
  float *b, *d, *h, *f0, *f1, *f2, *f3;
  // own row r: b, d, f0, f1, f3 at r * W; h and f2 at (r + 1) * W
};

// Outflow of one cell, flowUpdate.comp:34-62.  Channel pairs in packed
// f32x2 operations (lane by lane the same IEEE operations); packed products
// are summed with scalar adds, which the assembler does not contract.
template <bool F16>
__device__ __forceinline__ float4 outflow(const ResPlanes& p, const StepArgs& a, int W, int H,
                                          int r, int x, int y) {
  const int i = r * W + x, j = i + W;  // j: the cell in the planes with a ghost row above
  const float hc = p.h[j];
  const float2 hc2 = make_float2(hc, hc);
  const float2 ex = fsub2(hc2, make_float2(x + 1 < W ? p.h[j + 1] : 0.0f,    // (+x, -x)
                                           x > 0 ? p.h[j - 1] : 0.0f));
  const float2 ey = fsub2(hc2, make_float2(p.h[j + W], p.h[j - W]));        // (+y, -y)
  const float dc = p.d[i];
  const float2 kf2 = make_float2(a.kf, a.kf), ka2 = make_float2(a.ka, a.ka);
  const float2 px = fmul2(make_float2(p.f0[i], p.f1[i]), kf2), qx = fmul2(ex, ka2);
  const float2 py = fmul2(make_float2(p.f2[j], p.f3[i]), kf2), qy = fmul2(ey, ka2);
  float2 nx = make_float2(max0_fast(fadd(px.x, qx.x)), max0_fast(fadd(px.y, qx.y)));
  float2 ny = make_float2(max0_fast(fadd(py.x, qy.x)), max0_fast(fadd(py.y, qy.y)));
  if (a.closed) {
    if (x + 1 >= W) nx.x = 0.0f;
    if (x == 0) nx.y = 0.0f;
    if (y + 1 >= H) ny.x = 0.0f;
    if (y == 0) ny.y = 0.0f;
  }
  const float total = fmul(fadd(fadd(fadd(nx.x, nx.y), ny.x), ny.y), a.c);
  if (total > dc) {
    const float sc = scale_factor(dc, total);
    const float2 sc2 = make_float2(sc, sc);
    nx = fmul2(nx, sc2);
    ny = fmul2(ny, sc2);
  }
  if (F16) {
    const float2 fs2 = make_float2(a.flux_scale, a.flux_scale);
    const float2 fi2 = make_float2(a.flux_inv_scale, a.flux_inv_scale);
    nx = quantize_f16x2(nx, fs2, fi2);
    ny = quantize_f16x2(ny, fs2, fi2);
  }
  return make_float4(nx.x, nx.y, ny.x, ny.y);
}

__device__ __forceinline__ void store_outflow(const ResPlanes& p, int W, int r, int x,
                                              float4 n) {
  const int i = r * W + x;
  p.f0[i] = n.x;
  p.f1[i] = n.y;
  p.f2[i + W] = n.z;
  p.f3[i] = n.w;
}

// Depth of one cell, flowApply.comp:32-41, with the neighbours' channels it
// read (the flow vector, lines 45-46, is formed from them on the last step).
struct Applied {
  float4 fo;
  float X1, X0, Y1, Y0;
  float d;
};

__device__ __forceinline__ Applied apply(const ResPlanes& p, const StepArgs& a, int W, int r,
                                         int x) {
  const int i = r * W + x, j = i + W;
  Applied o;
  o.fo = make_float4(p.f0[i], p.f1[i], p.f2[j], p.f3[i]);
  o.X1 = x + 1 < W ? p.f1[i + 1] : 0.0f;  // -x outflow of the +x neighbour
  o.X0 = x > 0 ? p.f0[i - 1] : 0.0f;      // +x outflow of the -x neighbour
  o.Y1 = p.f3[i + W];                     // -y outflow of the +y neighbour
  o.Y0 = p.f2[i];                         // +y outflow of the -y neighbour
  // (inflow, outflow) side by side, each in the shader's order
  float2 io = fadd2(make_float2(o.X1, o.fo.x), make_float2(o.X0, o.fo.y));
  io = fadd2(io, make_float2(o.Y1, o.fo.z));
  io = fadd2(io, make_float2(o.Y0, o.fo.w));
  o.d = max0_fast(fadd(p.d[i], fmul(fsub(io.x, io.y), a.c)));
  return o;
}

template <bool F16>
__global__ void __launch_bounds__(kResThreads, 1)
    resident_kernel(const float* __restrict__ b_g, const float* __restrict__ d_g,
                    const void* __restrict__ f_g, const __grid_constant__ StepArgs a, int nsteps,
                    int R, int tpr) {
  extern __shared__ float4 res_smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int ncta = (int)cluster.num_blocks();
  const int W = a.W, H = a.H, pitch = a.pitch;
  const int y0 = rank * R;
  const int rows = max(0, min(R, H - y0));
  float* sm = reinterpret_cast<float*>(res_smem);
  ResPlanes p;
  p.b = sm;
  p.d = p.b + R * W;
  p.h = p.d + R * W;
  p.f0 = p.h + (R + 2) * W;
  p.f1 = p.f0 + R * W;
  p.f2 = p.f1 + R * W;
  p.f3 = p.f2 + (R + 1) * W;
  // threads: tpr per row (a power of two), kResThreads / tpr rows at a time
  const int tx = threadIdx.x & (tpr - 1);
  const int ty = threadIdx.x / tpr;
  const int ry = kResThreads / tpr;
  auto sync_all = [&]() {
    if (ncta > 1)
      cluster.sync();
    else
      __syncthreads();
  };

  // The adjacent CTAs' ghost rows that this CTA's edge rows feed: each CTA
  // writes its first and last rows of h (after the depth phase) and of the
  // -y / +y outflow (after the outflow phase) straight into its neighbours'
  // ghost rows through distributed shared memory.  A neighbour reads those
  // ghost rows only in the next phase, after the cluster barrier, and had
  // read their previous values before the barrier that ends its own previous
  // phase.  Ghost rows without a neighbour stay zero.
  const bool has_up = rank > 0 && rows > 0;
  const bool has_down = rows == R && y0 + R < H && rank + 1 < ncta;
  float* up_hg = has_up ? cluster.map_shared_rank(p.h + (R + 1) * W, rank - 1) : nullptr;
  float* up_f3g = has_up ? cluster.map_shared_rank(p.f3 + R * W, rank - 1) : nullptr;
  float* dn_hg = has_down ? cluster.map_shared_rank(p.h, rank + 1) : nullptr;
  float* dn_f2g = has_down ? cluster.map_shared_rank(p.f2, rank + 1) : nullptr;
  auto push_h = [&](int r, int x, float h) {
    if (r == 0 && has_up) up_hg[x] = h;
    if (r == rows - 1 && has_down) dn_hg[x] = h;
  };
  auto push_f = [&](int r, int x, float4 n) {
    if (r == 0 && has_up) up_f3g[x] = n.w;
    if (r == rows - 1 && has_down) dn_f2g[x] = n.z;
  };

  // sources that reach this CTA's rows, and the union of their boxes
  uint32_t mask = 0;
  int ux0 = INT_MAX, ux1 = INT_MIN, uy0 = INT_MAX, uy1 = INT_MIN;
  for (int k = 0; k < a.nsrc; ++k) {
    const DevSource& s = a.src[k];
    if (rows > 0 && s.by1 >= y0 && s.by0 <= y0 + rows - 1 && s.bx1 >= 0 && s.bx0 <= W - 1) {
      mask |= 1u << k;
      ux0 = min(ux0, s.bx0);
      ux1 = max(ux1, s.bx1);
      uy0 = min(uy0, s.by0);
      uy1 = max(uy1, s.by1);
    }
  }
  auto sources = [&](float d, int x, int y) {
    if (mask != 0u && x >= ux0 && x <= ux1 && y >= uy0 && y <= uy1)
      d = add_sources_inline(d, x, y, a, mask);
    return d;
  };

  // zero every plane (ghost rows and the unused rows of a partial CTA
  // included) in every CTA before any CTA writes a neighbour's ghost row,
  // then load the state, the first step's sources and h = d + b
  const int total = (int)res_floats(R, W);
  for (int k = threadIdx.x; k < total; k += kResThreads) sm[k] = 0.0f;
  sync_all();
  for (int r = ty; r < rows; r += ry) {
    const int y = y0 + r;
    for (int x = tx; x < W; x += tpr) {
      const size_t g = (size_t)y * pitch + x;
      const int i = r * W + x;
      float4 f;
      if (F16) {
        const uint2 raw = __ldg(reinterpret_cast<const uint2*>(f_g) + g);
        const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&raw.x));
        const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&raw.y));
        f = make_float4(fmul(lo.x, a.flux_inv_scale), fmul(lo.y, a.flux_inv_scale),
                        fmul(hi.x, a.flux_inv_scale), fmul(hi.y, a.flux_inv_scale));
      } else {
        f = __ldg(reinterpret_cast<const float4*>(f_g) + g);
      }
      p.f0[i] = f.x;
      p.f1[i] = f.y;
      p.f2[i + W] = f.z;
      p.f3[i] = f.w;
      const float b = __ldg(b_g + g);
      const float d = sources(__ldg(d_g + g), x, y);
      const float h = fadd(d, b);
      p.b[i] = b;
      p.d[i] = d;
      p.h[i + W] = h;
      push_h(r, x, h);
    }
  }
  sync_all();

  for (int step = 0; step < nsteps; ++step) {
    // outflow (each cell reads and writes only its own flux); two cells per
    // thread in flight where the thread has two
    for (int r = ty; r < rows; r += 2 * ry) {
      const int r2 = r + ry;
      for (int x = tx; x < W; x += tpr) {
        if (r2 < rows) {
          const float4 n1 = outflow<F16>(p, a, W, H, r, x, y0 + r);
          const float4 n2 = outflow<F16>(p, a, W, H, r2, x, y0 + r2);
          store_outflow(p, W, r, x, n1);
          store_outflow(p, W, r2, x, n2);
          push_f(r, x, n1);
          push_f(r2, x, n2);
        } else {
          const float4 n1 = outflow<F16>(p, a, W, H, r, x, y0 + r);
          store_outflow(p, W, r, x, n1);
          push_f(r, x, n1);
        }
      }
    }
    sync_all();

    // depth and flow map (each cell writes only its own depth)
    const bool last = step + 1 == nsteps;
    auto finish = [&](const Applied& o, int rr, int x) {
      const int y = y0 + rr;
      if (last) {
        const size_t g = (size_t)y * pitch + x;
        a.d_out[g] = o.d;
        if (F16) {
          const float2 fs2 = make_float2(a.flux_scale, a.flux_scale);
          const __half2 lo = __float22half2_rn(fmul2(make_float2(o.fo.x, o.fo.y), fs2));
          const __half2 hi = __float22half2_rn(fmul2(make_float2(o.fo.z, o.fo.w), fs2));
          uint2 packed;
          packed.x = *reinterpret_cast<const uint32_t*>(&lo);
          packed.y = *reinterpret_cast<const uint32_t*>(&hi);
          reinterpret_cast<uint2*>(a.f_out)[g] = packed;
        } else {
          reinterpret_cast<float4*>(a.f_out)[g] = o.fo;
        }
        a.v_out[g] = fsub2(fsub2(make_float2(o.X1, o.Y1), make_float2(o.fo.x, o.fo.z)),
                           fsub2(make_float2(o.X0, o.Y0), make_float2(o.fo.y, o.fo.w)));
      } else {
        const int i = rr * W + x;
        const float d = sources(o.d, x, y);
        const float h = fadd(d, p.b[i]);
        p.d[i] = d;
        p.h[i + W] = h;
        push_h(rr, x, h);
      }
    };
    for (int r = ty; r < rows; r += 2 * ry) {
      const int r2 = r + ry;
      for (int x = tx; x < W; x += tpr) {
        if (r2 < rows) {
          const Applied o1 = apply(p, a, W, r, x);
          const Applied o2 = apply(p, a, W, r2, x);
          finish(o1, r, x);
          finish(o2, r2, x);
        } else {
          finish(apply(p, a, W, r, x), r, x);
        }
      }
    }
    // the next phase reads what this one wrote, here and in the neighbours;
    // after the last step no CTA leaves while a neighbour may still write
    // into its ghost rows
    sync_all();
  }
}

struct ResidentShape {
  int cluster;  // CTAs
  int rows;     // rows per CTA
  int tpr;      // threads per row
  size_t smem;  // dynamic shared memory per CTA
};

int max_optin_smem() {
  static int v = -1;
  if (v < 0) {
    int dev = 0, s = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&s, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
      cudaGetLastError();
      s = 0;
    }
    v = s;
  }
  return v;
}

// ctas: the cluster size (1, 2, 4, 8 or 16), or 0 for the automatic choice,
// measured on GB300 for 32^2 to 512 x 128 grids: one CTA for at most 1024
// cells (one per thread: a block barrier is cheaper than a cluster barrier),
// else as many CTAs as the grid has rows, up to 16 (the per-step time falls
// with the cells per CTA faster than the cluster barrier grows).
bool resident_shape(int W, int H, int ctas, ResidentShape* out) {
  if (W < 1 || H < 1) return false;
  if (ctas != 0 && (ctas < 1 || ctas > kResidentMaxCluster || (ctas & (ctas - 1)) != 0))
    return false;
  const size_t limit = (size_t)max_optin_smem();
  auto smem_for = [&](int cs) {
    const int R = (H + cs - 1) / cs;
    return res_floats(R, W) * sizeof(float);
  };
  int cs = ctas;
  if (cs == 0) {
    cs = 1;
    if ((long long)W * H > kResThreads)
      while (cs < kResidentMaxCluster && cs * 2 <= H) cs <<= 1;
    while (cs < kResidentMaxCluster && smem_for(cs) > limit) cs <<= 1;
  }
  if (smem_for(cs) > limit) return false;
  int tpr = 32;
  while (tpr < W && tpr < kResThreads) tpr <<= 1;
  *out = {cs, (H + cs - 1) / cs, tpr, smem_for(cs)};
  return true;
}

const void* resident_fn(int flux_storage) {
  return flux_storage == TWS_FLUX_F16 ? (const void*)&resident_kernel<true>
                                      : (const void*)&resident_kernel<false>;
}

cudaLaunchConfig_t resident_config(const ResidentShape& sh, cudaLaunchAttribute* attr,
                                   cudaStream_t s) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)sh.cluster, 1, 1);
  cfg.blockDim = dim3(kResThreads, 1, 1);
  cfg.dynamicSmemBytes = sh.smem;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)sh.cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

}  // namespace

cudaError_t resident_supported(int W, int H, int flux_storage, int ctas, int* chosen) {
  ResidentShape sh;
  if (!resident_shape(W, H, ctas, &sh)) return cudaErrorNotSupported;
  const void* fn = resident_fn(flux_storage);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)max_optin_smem());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = resident_config(sh, attr, nullptr);
  int clusters = 0;
  e = cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg);
  if (e != cudaSuccess) return e;
  if (clusters < 1) return cudaErrorNotSupported;
  if (chosen) *chosen = sh.cluster;
  return cudaSuccess;
}

cudaError_t launch_resident(int flux_storage, int ctas, const float* b, const float* d,
                            const void* f, const StepArgs& a, int nsteps, cudaStream_t s) {
  ResidentShape sh;
  if (nsteps < 1 || nsteps > kResidentMaxSteps || ctas < 1 ||
      !resident_shape(a.W, a.H, ctas, &sh))
    return cudaErrorInvalidValue;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = resident_config(sh, attr, s);
  cudaError_t e;
  if (flux_storage == TWS_FLUX_F16)
    e = cudaLaunchKernelEx(&cfg, resident_kernel<true>, b, d, f, a, nsteps, sh.rows, sh.tpr);
  else
    e = cudaLaunchKernelEx(&cfg, resident_kernel<false>, b, d, f, a, nsteps, sh.rows, sh.tpr);
  count_launch();
  return e;
}

}  // namespace tws
