// tws_export.cu -- what the renderer reads from the simulation, on the device.
//
// * surface_kernel: the water shaders' per-texel arithmetic on the step's
//   outputs, written to plain device buffers (no graphics API):
//     surface height d + b                     waterRender.vert:23
//     dry mask d < 0.1                         waterRender.vert:22
//     tessellated height (d + b) - 0.1, and 10 lower where dry
//                                              waterRender.eval:33-35
//     heightmap normal from the 4 neighbour surface heights, sampled through
//     a REPEAT sampler (Terrain.cpp:313, 112-113)  waterRender.frag:50-62
//     flow speed |flow| and foam blend saturate(|flow|^2 * 0.00004) from the
//     RG16F flow map                           waterRender.frag:217,240-241,341,346
// * export kernels: the reference's texture layouts -- TerrainData as RGBA32F
//   (.r terrain, .g .b 0.3, .a depth; Terrain.cpp:216-220) with the 2x2 box
//   mip pyramid glGenerateMipmap builds after the steps (Terrain.cpp:273-276),
//   and the FlowMap as RG16F (flowApply.comp:7).
// Arithmetic is IEEE round-to-nearest without contraction; `normalize` is
// v / sqrt(dot(v, v)) and the mip filter ((a + b) + (c + d)) * 0.25 per
// channel (the GL specification leaves both to the implementation).

#include "tws_device.cuh"
#include "tws_internal.h"

namespace tws {
namespace {

__device__ __forceinline__ float surf(const float* b, const float* d, size_t i) {
  return fadd(d[i], b[i]);
}

__device__ __forceinline__ float half_round(float v) { return __half2float(__float2half_rn(v)); }

// cross((0, A, 1), (1, B, 0)) evaluated component by component as GLSL
// defines cross(x, y) = (x1 y2 - y1 x2, x2 y0 - y2 x0, x0 y1 - y0 x1)
// (waterRender.frag:63-65): (A*0 - B*1, 1*1 - 0*0, 0*B - 1*A) = (A*0 - B, 1,
// 0*B - A).  The products with zero keep the sign of zero a flat surface
// gives (A = 0 or B = 0), which -B and -A alone would flip.
__device__ __forceinline__ void heightmap_cross(float A, float B, float& nx, float& ny,
                                                float& nz) {
  nx = fsub(fmul(A, 0.0f), B);
  ny = 1.0f;
  nz = fsub(fmul(0.0f, B), A);
}

__global__ void surface_kernel(const float* __restrict__ b, const float* __restrict__ d,
                               const float2* __restrict__ v, int W, int H, int pitch,
                               tws_surface_out o) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t i = (size_t)y * pitch + x;
  const size_t out = (size_t)y * W + x;
  const float dc = d[i];
  const float h = surf(b, d, i);
  if (o.height) o.height[out] = h;
  if (o.dry) o.dry[out] = dc < 0.1f ? 1 : 0;
  if (o.render_height) {
    float t = fsub(h, 0.1f);
    if (dc < 0.1f) t = fsub(t, 10.0f);
    o.render_height[out] = t;
  }
  if (o.normal) {
    const int xm = x == 0 ? W - 1 : x - 1, xp = x + 1 == W ? 0 : x + 1;
    const int ym = y == 0 ? H - 1 : y - 1, yp = y + 1 == H ? 0 : y + 1;
    const float h0 = surf(b, d, (size_t)ym * pitch + x);
    const float h1 = surf(b, d, (size_t)yp * pitch + x);
    const float h2 = surf(b, d, (size_t)y * pitch + xp);
    const float h3 = surf(b, d, (size_t)y * pitch + xm);
    const float A = fsub(h1, h0), B = fsub(h2, h3);
    float nx, ny, nz;
    heightmap_cross(A, B, nx, ny, nz);
    const float len = __fsqrt_rn(fadd(fadd(fmul(nx, nx), fmul(ny, ny)), fmul(nz, nz)));
    o.normal[3 * out + 0] = fdiv(nx, len);
    o.normal[3 * out + 1] = fdiv(ny, len);
    o.normal[3 * out + 2] = fdiv(nz, len);
  }
  if (o.flow_speed || o.foam) {
    const float2 fv = v[i];
    const float fx = half_round(fv.x), fy = half_round(fv.y);
    const float s2 = fadd(fmul(fx, fx), fmul(fy, fy));
    if (o.flow_speed) o.flow_speed[out] = __fsqrt_rn(s2);
    if (o.foam) o.foam[out] = saturate01(fmul(s2, 0.00004f));
  }
}

// The same per-texel arithmetic, four cells per thread for widths that are a
// multiple of 4: 16-byte loads and stores (the packed outputs' rows then start
// on 16-byte boundaries, and so do the pitched inputs' rows).
__global__ void surface_kernel4(const float* __restrict__ b, const float* __restrict__ d,
                                const float2* __restrict__ v, int W, int H, int pitch,
                                tws_surface_out o) {
  const int x = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t i = (size_t)y * pitch + x;
  const size_t out = (size_t)y * W + x;
  const float4 b4 = *reinterpret_cast<const float4*>(b + i);
  const float4 d4 = *reinterpret_cast<const float4*>(d + i);
  const float dc[4] = {d4.x, d4.y, d4.z, d4.w};
  const float h[4] = {fadd(d4.x, b4.x), fadd(d4.y, b4.y), fadd(d4.z, b4.z), fadd(d4.w, b4.w)};
  if (o.height) *reinterpret_cast<float4*>(o.height + out) = make_float4(h[0], h[1], h[2], h[3]);
  if (o.dry)
    *reinterpret_cast<uchar4*>(o.dry + out) =
        make_uchar4(dc[0] < 0.1f, dc[1] < 0.1f, dc[2] < 0.1f, dc[3] < 0.1f);
  if (o.render_height) {
    float t[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      t[k] = fsub(h[k], 0.1f);
      if (dc[k] < 0.1f) t[k] = fsub(t[k], 10.0f);
    }
    *reinterpret_cast<float4*>(o.render_height + out) = make_float4(t[0], t[1], t[2], t[3]);
  }
  if (o.normal) {
    const int ym = y == 0 ? H - 1 : y - 1, yp = y + 1 == H ? 0 : y + 1;
    const int xm = x == 0 ? W - 1 : x - 1, xp = x + 4 == W ? 0 : x + 4;
    const size_t iu = (size_t)ym * pitch + x, id = (size_t)yp * pitch + x;
    const float4 bu = *reinterpret_cast<const float4*>(b + iu);
    const float4 du = *reinterpret_cast<const float4*>(d + iu);
    const float4 bd = *reinterpret_cast<const float4*>(b + id);
    const float4 dd = *reinterpret_cast<const float4*>(d + id);
    const float hu[4] = {fadd(du.x, bu.x), fadd(du.y, bu.y), fadd(du.z, bu.z), fadd(du.w, bu.w)};
    const float hd[4] = {fadd(dd.x, bd.x), fadd(dd.y, bd.y), fadd(dd.z, bd.z), fadd(dd.w, bd.w)};
    const float hl = surf(b, d, (size_t)y * pitch + xm), hr = surf(b, d, (size_t)y * pitch + xp);
    float n[12];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float h2 = k < 3 ? h[k + 1] : hr, h3 = k > 0 ? h[k - 1] : hl;
      const float A = fsub(hd[k], hu[k]), B = fsub(h2, h3);
      float nx, ny, nz;
      heightmap_cross(A, B, nx, ny, nz);
      const float len = __fsqrt_rn(fadd(fadd(fmul(nx, nx), fmul(ny, ny)), fmul(nz, nz)));
      n[3 * k + 0] = fdiv(nx, len);
      n[3 * k + 1] = fdiv(ny, len);
      n[3 * k + 2] = fdiv(nz, len);
    }
    float4* no = reinterpret_cast<float4*>(o.normal + 3 * out);
    no[0] = make_float4(n[0], n[1], n[2], n[3]);
    no[1] = make_float4(n[4], n[5], n[6], n[7]);
    no[2] = make_float4(n[8], n[9], n[10], n[11]);
  }
  if (o.flow_speed || o.foam) {
    const float4 v01 = *reinterpret_cast<const float4*>(v + i);
    const float4 v23 = *reinterpret_cast<const float4*>(v + i + 2);
    const float vx[4] = {v01.x, v01.z, v23.x, v23.z}, vy[4] = {v01.y, v01.w, v23.y, v23.w};
    float sp[4], fo[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float fx = half_round(vx[k]), fy = half_round(vy[k]);
      const float s2 = fadd(fmul(fx, fx), fmul(fy, fy));
      sp[k] = __fsqrt_rn(s2);
      fo[k] = saturate01(fmul(s2, 0.00004f));
    }
    if (o.flow_speed)
      *reinterpret_cast<float4*>(o.flow_speed + out) = make_float4(sp[0], sp[1], sp[2], sp[3]);
    if (o.foam) *reinterpret_cast<float4*>(o.foam + out) = make_float4(fo[0], fo[1], fo[2], fo[3]);
  }
}

// TerrainData (RGBA32F) and the RG16F flow map in one pass, four cells per
// thread, for widths that are a multiple of 4 (either output may be null).
__global__ void export_kernel4(const float* __restrict__ b, const float* __restrict__ d,
                               const float2* __restrict__ v, int W, int H, int pitch,
                               float4* __restrict__ rgba, __half2* __restrict__ flowmap) {
  const int x = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t i = (size_t)y * pitch + x;
  const size_t out = (size_t)y * W + x;
  if (rgba) {
    const float4 b4 = *reinterpret_cast<const float4*>(b + i);
    const float4 d4 = *reinterpret_cast<const float4*>(d + i);
    rgba[out + 0] = make_float4(b4.x, 0.3f, 0.3f, d4.x);
    rgba[out + 1] = make_float4(b4.y, 0.3f, 0.3f, d4.y);
    rgba[out + 2] = make_float4(b4.z, 0.3f, 0.3f, d4.z);
    rgba[out + 3] = make_float4(b4.w, 0.3f, 0.3f, d4.w);
  }
  if (flowmap) {
    const float4 v01 = *reinterpret_cast<const float4*>(v + i);
    const float4 v23 = *reinterpret_cast<const float4*>(v + i + 2);
    const __half2 h0 = __floats2half2_rn(v01.x, v01.y), h1 = __floats2half2_rn(v01.z, v01.w);
    const __half2 h2 = __floats2half2_rn(v23.x, v23.y), h3 = __floats2half2_rn(v23.z, v23.w);
    uint4 packed;
    packed.x = *reinterpret_cast<const uint32_t*>(&h0);
    packed.y = *reinterpret_cast<const uint32_t*>(&h1);
    packed.z = *reinterpret_cast<const uint32_t*>(&h2);
    packed.w = *reinterpret_cast<const uint32_t*>(&h3);
    *reinterpret_cast<uint4*>(flowmap + out) = packed;
  }
}

__global__ void terrain_rgba_kernel(const float* __restrict__ b, const float* __restrict__ d,
                                    int W, int H, int pitch, float4* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t i = (size_t)y * pitch + x;
  out[(size_t)y * W + x] = make_float4(b[i], 0.3f, 0.3f, d[i]);
}

__global__ void flowmap_kernel(const float2* __restrict__ v, int W, int H, int pitch,
                               __half2* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const float2 fv = v[(size_t)y * pitch + x];
  out[(size_t)y * W + x] = __floats2half2_rn(fv.x, fv.y);
}

__device__ __forceinline__ float avg4(float a, float b, float c, float d) {
  return fmul(fadd(fadd(a, b), fadd(c, d)), 0.25f);
}

// Up to kMipChain levels of the mip pyramid in one launch.  A CTA takes a
// 32 x 32 texel block of the source level: each thread filters a 2 x 2 quad
// of it into the first level in registers, and the CTA halves that in shared
// memory level by level with the 2 x 2 filter ((a + b) + (c + e)) * 0.25 (a, b the
// upper texel pair, c, e the lower), writing each level's texels of
// the block.  Level l + m texel q depends only on source texels
// [q 2^m, (q + 1) 2^m), so every texel of a level of floor(w / 2^m) texels
// is made from texels of this block inside the source; texels past a
// level's edge are computed from zero fill and not written.
constexpr int kMipBlock = 32;
constexpr int kMipChain = 5;  // 32 -> 16 -> 8 -> 4 -> 2 -> 1
struct MipChain {
  float4* dst[kMipChain];
  int w[kMipChain], h[kMipChain];  // sizes of the levels written
  int n;                           // levels written, 1 .. kMipChain
};

__global__ void __launch_bounds__(256)
    mip_chain_kernel(const float4* __restrict__ src, int sw, int sh, MipChain c) {
  constexpr int Q = kMipBlock / 2;  // the first level's texels per block side
  __shared__ float4 buf[2][Q * Q];
  const int bx = blockIdx.x * kMipBlock, by = blockIdx.y * kMipBlock;
  const int tid = threadIdx.x;
  {
    // the first level: each thread filters its 2 x 2 source texels in
    // registers (texels past the source's edge read as zero; the output they
    // feed is past the level's edge and not written)
    const int qx = tid % Q, qy = tid / Q;
    const int x = bx + 2 * qx, y = by + 2 * qy;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    auto at = [&](int xx, int yy) {
      return (xx < sw && yy < sh) ? src[(size_t)yy * sw + xx] : z;
    };
    const float4 a = at(x, y), b = at(x + 1, y), cc = at(x, y + 1), e = at(x + 1, y + 1);
    const float4 r = make_float4(avg4(a.x, b.x, cc.x, e.x), avg4(a.y, b.y, cc.y, e.y),
                                 avg4(a.z, b.z, cc.z, e.z), avg4(a.w, b.w, cc.w, e.w));
    buf[0][qy * Q + qx] = r;
    const int gx = (bx >> 1) + qx, gy = (by >> 1) + qy;
    if (gx < c.w[0] && gy < c.h[0]) c.dst[0][(size_t)gy * c.w[0] + gx] = r;
  }
  __syncthreads();
  // unrolled so that every level index is a constant (an indexed kernel
  // parameter would be copied to local memory)
#pragma unroll
  for (int l = 1; l < kMipChain; ++l) {
    if (l >= c.n) break;  // the same for every thread
    const int side = Q >> (l - 1), half = side / 2;
    const float4* in = buf[(l - 1) & 1];
    float4* out = buf[l & 1];
    const int ox = bx >> (l + 1), oy = by >> (l + 1);  // the block's origin in this level
    for (int i = tid; i < half * half; i += blockDim.x) {
      const int x = i % half, y = i / half;
      const float4 a = in[(2 * y) * side + 2 * x], b = in[(2 * y) * side + 2 * x + 1];
      const float4 cc = in[(2 * y + 1) * side + 2 * x], e = in[(2 * y + 1) * side + 2 * x + 1];
      const float4 r = make_float4(avg4(a.x, b.x, cc.x, e.x), avg4(a.y, b.y, cc.y, e.y),
                                   avg4(a.z, b.z, cc.z, e.z), avg4(a.w, b.w, cc.w, e.w));
      out[y * half + x] = r;
      const int gx = ox + x, gy = oy + y;
      if (gx < c.w[l] && gy < c.h[l]) c.dst[l][(size_t)gy * c.w[l] + gx] = r;
    }
    __syncthreads();
  }
}

// export_kernel4's work for a 64 x 64 block of cells (W % 4 == 0, H even)
// plus up to six mip levels of the block (32 x 32 texels down to 1 x 1): each
// thread exports two 4 x 2 patches and filters each into two level-1 texels
// in registers, and the CTA halves level 1 in shared memory down to the last
// level, with the filter of mip_chain_kernel.  Texels past a level's edge are
// computed from zero fill and not written; level-1 texels inside the level
// use only cells on the grid.
constexpr int kMipFused = 6;  // 64 -> 32 -> 16 -> 8 -> 4 -> 2 -> 1
struct MipLevels {
  float4* dst[kMipFused];
  int w[kMipFused], h[kMipFused];  // sizes of the levels written
  int n;                           // levels written, 1 .. kMipFused
};

__global__ void __launch_bounds__(256)
    export_mips_kernel4(const float* __restrict__ b, const float* __restrict__ d,
                        const float2* __restrict__ v, int W, int H, int pitch,
                        float4* __restrict__ rgba, __half2* __restrict__ flowmap, MipLevels m) {
  constexpr int Q = 32;  // level-1 texels per block side
  __shared__ float4 buf[2][Q * Q];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 x 16 threads
  const int bx = blockIdx.x * 64, by = blockIdx.y * 64;
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    // cells (x .. x + 3, y .. y + 1); level-1 texels (x/2, x/2 + 1) of row y/2
    const int x = bx + 4 * tx, y = by + 4 * ty + 2 * half;
    float4 t[2][4];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      if (x < W && y + r < H) {
        const size_t i = (size_t)(y + r) * pitch + x;
        const size_t out = (size_t)(y + r) * W + x;
        const float4 b4 = *reinterpret_cast<const float4*>(b + i);
        const float4 d4 = *reinterpret_cast<const float4*>(d + i);
        t[r][0] = make_float4(b4.x, 0.3f, 0.3f, d4.x);
        t[r][1] = make_float4(b4.y, 0.3f, 0.3f, d4.y);
        t[r][2] = make_float4(b4.z, 0.3f, 0.3f, d4.z);
        t[r][3] = make_float4(b4.w, 0.3f, 0.3f, d4.w);
#pragma unroll
        for (int k = 0; k < 4; ++k) rgba[out + k] = t[r][k];
        if (flowmap) {
          const float4 v01 = *reinterpret_cast<const float4*>(v + i);
          const float4 v23 = *reinterpret_cast<const float4*>(v + i + 2);
          const __half2 h0 = __floats2half2_rn(v01.x, v01.y);
          const __half2 h1 = __floats2half2_rn(v01.z, v01.w);
          const __half2 h2 = __floats2half2_rn(v23.x, v23.y);
          const __half2 h3 = __floats2half2_rn(v23.z, v23.w);
          uint4 packed;
          packed.x = *reinterpret_cast<const uint32_t*>(&h0);
          packed.y = *reinterpret_cast<const uint32_t*>(&h1);
          packed.z = *reinterpret_cast<const uint32_t*>(&h2);
          packed.w = *reinterpret_cast<const uint32_t*>(&h3);
          *reinterpret_cast<uint4*>(flowmap + out) = packed;
        }
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) t[r][k] = z;
      }
    }
    const int qy = 2 * ty + half, gy = (by >> 1) + qy;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const float4 a = t[0][2 * j], c0 = t[0][2 * j + 1], c = t[1][2 * j], e = t[1][2 * j + 1];
      const float4 r = make_float4(avg4(a.x, c0.x, c.x, e.x), avg4(a.y, c0.y, c.y, e.y),
                                   avg4(a.z, c0.z, c.z, e.z), avg4(a.w, c0.w, c.w, e.w));
      const int qx = 2 * tx + j, gx = (bx >> 1) + qx;
      buf[0][qy * Q + qx] = r;
      if (gx < m.w[0] && gy < m.h[0]) m.dst[0][(size_t)gy * m.w[0] + gx] = r;
    }
  }
  __syncthreads();
  // levels 2 .. m.n, unrolled so that every level index is a constant (an
  // indexed kernel parameter would be copied to local memory)
#pragma unroll
  for (int l = 1; l < kMipFused; ++l) {
    if (l >= m.n) break;  // the same for every thread
    const int side = Q >> (l - 1), half = side / 2;
    const float4* in = buf[(l - 1) & 1];
    float4* out = buf[l & 1];
    const int ox = bx >> (l + 1), oy = by >> (l + 1);  // the block's origin in this level
    for (int i = threadIdx.x; i < half * half; i += blockDim.x) {
      const int x = i % half, y = i / half;
      const float4 a = in[(2 * y) * side + 2 * x], c0 = in[(2 * y) * side + 2 * x + 1];
      const float4 c = in[(2 * y + 1) * side + 2 * x], e = in[(2 * y + 1) * side + 2 * x + 1];
      const float4 r = make_float4(avg4(a.x, c0.x, c.x, e.x), avg4(a.y, c0.y, c.y, e.y),
                                   avg4(a.z, c0.z, c.z, e.z), avg4(a.w, c0.w, c.w, e.w));
      out[y * half + x] = r;
      const int gx = ox + x, gy = oy + y;
      if (gx < m.w[l] && gy < m.h[l]) m.dst[l][(size_t)gy * m.w[l] + gx] = r;
    }
    __syncthreads();
  }
}

dim3 grid2d(int w, int h) { return dim3((w + 31) / 32, (h + 7) / 8); }

}  // namespace

// The four-cell kernels need W % 4 == 0 and every caller-owned output on a
// 16-byte boundary (the dry mask on a 4-byte one); the library's own inputs
// always are (256-byte aligned buffers, pitch a multiple of 32).
static bool aligned(const void* p, uintptr_t a) {
  return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0;
}

cudaError_t launch_surface(const float* b, const float* d, const float2* v, int W, int H,
                           int pitch, const tws_surface_out& o, cudaStream_t s) {
  const bool wide = W % 4 == 0 && aligned(o.height, 16) && aligned(o.render_height, 16) &&
                    aligned(o.normal, 16) && aligned(o.flow_speed, 16) && aligned(o.foam, 16) &&
                    aligned(o.dry, 4);
  if (wide)
    surface_kernel4<<<grid2d(W / 4, H), dim3(32, 8), 0, s>>>(b, d, v, W, H, pitch, o);
  else
    surface_kernel<<<grid2d(W, H), dim3(32, 8), 0, s>>>(b, d, v, W, H, pitch, o);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_export(const float* b, const float* d, const float2* v, int W, int H,
                          int pitch, float* terrain_rgba, uint16_t* flowmap, int mip_levels,
                          float* mips, cudaStream_t s) {
  const bool wide = W % 4 == 0 && aligned(terrain_rgba, 16) && aligned(flowmap, 16);
  // with mips, the first level comes out of the same pass (even heights)
  const bool fuse_mip1 = wide && terrain_rgba && mips && mip_levels >= 1 && H % 2 == 0;
  MipLevels fused{};
  if (fuse_mip1) {
    // the export and up to six mip levels in one pass
    float4* p = reinterpret_cast<float4*>(mips);
    int w = W, h = H;
    while (fused.n < kMipFused && fused.n < mip_levels && w >= 2 && h >= 2) {
      w /= 2;
      h /= 2;
      fused.dst[fused.n] = p;
      fused.w[fused.n] = w;
      fused.h[fused.n] = h;
      p += (size_t)w * h;
      ++fused.n;
    }
    export_mips_kernel4<<<dim3((W + 63) / 64, (H + 63) / 64), 256, 0, s>>>(
        b, d, v, W, H, pitch, reinterpret_cast<float4*>(terrain_rgba),
        reinterpret_cast<__half2*>(flowmap), fused);
    count_launch();
  } else if (wide && (flowmap || terrain_rgba)) {
    export_kernel4<<<grid2d(W / 4, H), dim3(32, 8), 0, s>>>(
        b, d, v, W, H, pitch, reinterpret_cast<float4*>(terrain_rgba),
        reinterpret_cast<__half2*>(flowmap));
    count_launch();
  } else {
    if (flowmap) {
      flowmap_kernel<<<grid2d(W, H), dim3(32, 8), 0, s>>>(v, W, H, pitch,
                                                           reinterpret_cast<__half2*>(flowmap));
      count_launch();
    }
    if (terrain_rgba) {
      terrain_rgba_kernel<<<grid2d(W, H), dim3(32, 8), 0, s>>>(
          b, d, W, H, pitch, reinterpret_cast<float4*>(terrain_rgba));
      count_launch();
    }
  }
  if (terrain_rgba && mips) {
    const float4* src = reinterpret_cast<const float4*>(terrain_rgba);
    float4* dst = reinterpret_cast<float4*>(mips);
    int sw = W, sh = H, l = 1;
    if (fuse_mip1) {  // levels 1 .. fused.n are written; continue from the last
      src = fused.dst[fused.n - 1];
      dst = fused.dst[fused.n - 1] + (size_t)fused.w[fused.n - 1] * fused.h[fused.n - 1];
      sw = fused.w[fused.n - 1];
      sh = fused.h[fused.n - 1];
      l = fused.n + 1;
    }
    // the remaining levels, up to kMipChain per launch (4096^2: 2 launches
    // for levels 7..12)
    while (l <= mip_levels && sw >= 2 && sh >= 2) {
      MipChain c{};
      int w = sw, h = sh;
      float4* p = dst;
      while (c.n < kMipChain && l + c.n <= mip_levels && w >= 2 && h >= 2) {
        w /= 2;
        h /= 2;
        c.dst[c.n] = p;
        c.w[c.n] = w;
        c.h[c.n] = h;
        p += (size_t)w * h;
        ++c.n;
      }
      const dim3 grid((sw + kMipBlock - 1) / kMipBlock, (sh + kMipBlock - 1) / kMipBlock);
      mip_chain_kernel<<<grid, 256, 0, s>>>(src, sw, sh, c);
      count_launch();
      src = c.dst[c.n - 1];
      sw = c.w[c.n - 1];
      sh = c.h[c.n - 1];
      dst = p;
      l += c.n;
    }
  }
  return cudaGetLastError();
}

}  // namespace tws
