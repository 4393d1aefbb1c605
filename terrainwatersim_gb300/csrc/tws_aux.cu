// tws_aux.cu -- the kernels around the step: one-shot sources, the FP64 total
// volume, the synthetic scene generator and flux format conversion.

#include <algorithm>
#include <mutex>

#include "tws_device.cuh"
#include "tws_internal.h"

namespace tws {
namespace {

// ---- one-shot source (the reference's brush dispatch, Terrain.cpp:150-168) --
__global__ void apply_source_kernel(float* d, int W, int H, int pitch, StepArgs a) {
  const int gx = a.src[0].bx0 + blockIdx.x * blockDim.x + threadIdx.x;
  const int gy = a.src[0].by0 + blockIdx.y * blockDim.y + threadIdx.y;
  if (gx > a.src[0].bx1 || gy > a.src[0].by1 || gx >= W || gy >= H) return;
  const size_t g = (size_t)gy * pitch + gx;
  d[g] = add_sources(d[g], gx, gy, a, 1u);
}

// ---- total volume in FP64 ---------------------------------------------------
// Two passes with a fixed partition and a fixed reduction tree, so the result
// is deterministic for a given grid size.  Pass 1: block r sums rows
// r, r + gridDim.x, ... into partials[r].  Pass 2: one block sums partials.
constexpr int kVolThreads = 256;
constexpr int kVolMaxBlocks = 1024;

__device__ double block_sum(double v) {
  __shared__ double warp_part[kVolThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_part[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    s = lane < kVolThreads / 32 ? warp_part[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  return s;  // valid in thread 0
}

__global__ void __launch_bounds__(kVolThreads)
    volume_rows_kernel(const float* d, int W, int H, int pitch, double* partials) {
  double acc = 0.0;
  for (int y = blockIdx.x; y < H; y += gridDim.x) {
    const float* row = d + (size_t)y * pitch;
    for (int x = threadIdx.x; x < W; x += kVolThreads) acc += (double)row[x];
  }
  const double s = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kVolThreads)
    volume_final_kernel(const double* partials, int n, double cell_area, double* out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += kVolThreads) acc += partials[i];
  const double s = block_sum(acc);
  if (threadIdx.x == 0) *out = s * cell_area;
}

// ---- scene generator ----------------------------------------------------------
// Seeded PCG32 value noise, the definition the oracle's generator states:
// octave o (0..5) has lattice spacing 64 >> o; its lattice value (i, j) is
// output number j*Lx + i of the PCG32 stream (seed, o + 1), Lx = W/s + 2,
// mapped to [0, 1) with 24 bits; smoothstep-bilinear interpolation; octave
// amplitudes 1, 1/2, ...; sum / 1.96875 * height_scale.
// PCG32 is O'Neill's XSH-RR 64/32 generator; lattice points are generated in
// parallel by jumping the LCG ahead (Brown 1994).
constexpr int kOctaves = 6;
}  // namespace

constexpr uint64_t kPcgMult = 6364136223846793005ULL;

struct Pcg32 {
  uint64_t state, inc;
  __host__ __device__ void seed(uint64_t initstate, uint64_t initseq) {
    state = 0u;
    inc = (initseq << 1u) | 1u;
    next();
    state += initstate;
    next();
  }
  __host__ __device__ uint32_t next() {
    const uint64_t old = state;
    state = old * kPcgMult + inc;
    const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((0u - rot) & 31u));
  }
  __host__ __device__ void advance(uint64_t delta) {
    uint64_t cur_mult = kPcgMult, cur_plus = inc, acc_mult = 1u, acc_plus = 0u;
    while (delta > 0) {
      if (delta & 1u) {
        acc_mult *= cur_mult;
        acc_plus = acc_plus * cur_mult + cur_plus;
      }
      cur_plus = (cur_mult + 1u) * cur_plus;
      cur_mult *= cur_mult;
      delta >>= 1u;
    }
    state = acc_mult * state + acc_plus;
  }
};

namespace {

struct Lattice {
  float* v[kOctaves];
  int lx[kOctaves];
  long long n[kOctaves];
  uint64_t base_state[kOctaves], inc[kOctaves];
};

__global__ void lattice_kernel(Lattice L, int o) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= L.n[o]) return;
  Pcg32 g;
  g.state = L.base_state[o];
  g.inc = L.inc[o];
  g.advance((uint64_t)k);
  L.v[o][k] = (float)(g.next() >> 8) * (1.0f / 16777216.0f);
}

__device__ __forceinline__ float smooth01(float t) {
  return fmul(fmul(t, t), fsub(3.0f, fmul(2.0f, t)));
}
__device__ __forceinline__ float lerpf(float a, float b, float t) {
  return fadd(a, fmul(fsub(b, a), t));
}

__global__ void scene_kernel(Lattice L, int W, int H, int pitch, float height_scale, float fill,
                             float* b, float* d) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  float acc = 0.0f, amp = 1.0f;
#pragma unroll
  for (int o = 0; o < kOctaves; ++o) {
    const int s = 64 >> o;
    const float inv = 1.0f / (float)s;
    const int i = x / s, j = y / s;
    const float sx = smooth01(fmul((float)(x % s), inv));
    const float sy = smooth01(fmul((float)(y % s), inv));
    const float* V = L.v[o];
    const int Lx = L.lx[o];
    const float v00 = V[(size_t)j * Lx + i], v10 = V[(size_t)j * Lx + i + 1];
    const float v01 = V[(size_t)(j + 1) * Lx + i], v11 = V[(size_t)(j + 1) * Lx + i + 1];
    const float v = lerpf(lerpf(v00, v10, sx), lerpf(v01, v11, sx), sy);
    acc = fadd(acc, fmul(amp, v));
    amp = fmul(amp, 0.5f);
  }
  const float bb = fmul(fdiv(acc, 1.96875f), height_scale);
  const size_t g = (size_t)y * pitch + x;
  b[g] = bb;
  d[g] = max0(fsub(fill, bb));
}

// ---- flux format conversion -----------------------------------------------------
__global__ void flux_to_f32_kernel(const void* f, int f16, float inv_scale, int W, int H,
                                   int pitch, float4* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t g = (size_t)y * pitch + x;
  float4 r;
  if (f16) {
    const __half2* h = reinterpret_cast<const __half2*>(f) + 2 * g;
    const float2 lo = __half22float2(h[0]), hi = __half22float2(h[1]);
    r = make_float4(fmul(lo.x, inv_scale), fmul(lo.y, inv_scale), fmul(hi.x, inv_scale),
                    fmul(hi.y, inv_scale));
  } else {
    r = reinterpret_cast<const float4*>(f)[g];
  }
  out[(size_t)y * W + x] = r;
}

__global__ void flux_from_f32_kernel(const float4* in, int f16, float scale, int W, int H,
                                     int pitch, void* f) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t g = (size_t)y * pitch + x;
  const float4 v = in[(size_t)y * W + x];
  if (f16) {
    __half2* h = reinterpret_cast<__half2*>(f) + 2 * g;
    h[0] = __floats2half2_rn(fminf(fmul(v.x, scale), 65504.0f), fminf(fmul(v.y, scale), 65504.0f));
    h[1] = __floats2half2_rn(fminf(fmul(v.z, scale), 65504.0f), fminf(fmul(v.w, scale), 65504.0f));
  } else {
    reinterpret_cast<float4*>(f)[g] = v;
  }
}

// Rows of packed host-layout arrays to or from rows of the pitched state, up
// to four arrays in one launch (a null source clears its destination).  Each
// thread moves 16 bytes where both rows allow it, else 4.
__global__ void __launch_bounds__(256) stage_rows_kernel(StageRows sr, int H) {
  const unsigned stride = gridDim.x * blockDim.x;
  for (int a = 0; a < sr.n; ++a) {
    const int vec = sr.vec[a];  // floats per item: 4 or 1
    const unsigned per_row = (unsigned)(sr.row_floats[a] / vec);
    const unsigned items = per_row * (unsigned)H;
    const float* __restrict__ src = sr.src[a];
    float* __restrict__ dst = sr.dst[a];
    const size_t sp = (size_t)sr.src_pitch[a], dp = (size_t)sr.dst_pitch[a];
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < items; i += stride) {
      const unsigned y = i / per_row, x = (i - y * per_row) * vec;
      float* o = dst + y * dp + x;
      if (vec == 4) {
        const float4 v = src ? __ldcs(reinterpret_cast<const float4*>(src + y * sp + x))
                             : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        __stcs(reinterpret_cast<float4*>(o), v);
      } else {
        *o = src ? src[y * sp + x] : 0.0f;
      }
    }
  }
}

}  // namespace

cudaError_t launch_stage_rows(const StageRows& sr_in, int H, cudaStream_t st) {
  StageRows sr = sr_in;
  long long most = 0;
  for (int a = 0; a < sr.n; ++a) {
    const bool aligned = sr.row_floats[a] % 4 == 0 && sr.src_pitch[a] % 4 == 0 &&
                         sr.dst_pitch[a] % 4 == 0 &&
                         reinterpret_cast<uintptr_t>(sr.src[a]) % 16 == 0 &&
                         reinterpret_cast<uintptr_t>(sr.dst[a]) % 16 == 0;
    sr.vec[a] = aligned ? 4 : 1;
    const long long items = (long long)(sr.row_floats[a] / sr.vec[a]) * H;
    if (items > 0x7fffffffLL) return cudaErrorInvalidValue;  // 32-bit item index
    most = std::max(most, items);
  }
  if (most == 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    sms = 1;
  const long long blocks = std::min<long long>((most + 255) / 256, 8LL * sms);
  stage_rows_kernel<<<(unsigned)blocks, 256, 0, st>>>(sr, H);
  count_launch();
  return cudaGetLastError();
}

DevSource make_dev_source(const tws_source& s) {
  DevSource r{};
  r.kind = s.kind;
  r.cx = s.cx;
  r.cy = s.cy;
  r.radius = s.radius;
  r.rate = s.rate;
  if (s.kind == TWS_SOURCE_DISK) {
    r.icx = (int)s.cx;
    r.icy = (int)s.cy;
    r.ir = (int)s.radius;
    r.bx0 = r.icx - r.ir;
    r.bx1 = r.icx + r.ir;
    r.by0 = r.icy - r.ir;
    r.by1 = r.icy + r.ir;
  } else {
    // Every cell the brush can change satisfies |(x,y) - c|^2 < S (1 + eps);
    // the box is widened by two cells beyond sqrt(S).
    const float rr = sqrtf(s.radius > 0.0f ? s.radius : 0.0f);
    r.bx0 = (int)floorf(s.cx - rr) - 2;
    r.bx1 = (int)ceilf(s.cx + rr) + 2;
    r.by0 = (int)floorf(s.cy - rr) - 2;
    r.by1 = (int)ceilf(s.cy + rr) + 2;
  }
  return r;
}

cudaError_t launch_apply_source(float* d, int W, int H, int pitch, const DevSource& s,
                                cudaStream_t st) {
  StepArgs a{};
  a.nsrc = 1;
  a.src[0] = s;
  a.src[0].bx0 = std::max(0, s.bx0);
  a.src[0].by0 = std::max(0, s.by0);
  a.src[0].bx1 = std::min(W - 1, s.bx1);
  a.src[0].by1 = std::min(H - 1, s.by1);
  if (a.src[0].bx0 > a.src[0].bx1 || a.src[0].by0 > a.src[0].by1) return cudaSuccess;
  const int w = a.src[0].bx1 - a.src[0].bx0 + 1, h = a.src[0].by1 - a.src[0].by0 + 1;
  dim3 blk(32, 8), grd((w + 31) / 32, (h + 7) / 8);
  apply_source_kernel<<<grd, blk, 0, st>>>(d, W, H, pitch, a);
  count_launch();
  return cudaGetLastError();
}

int volume_partials_needed() { return kVolMaxBlocks; }

cudaError_t launch_volume(const float* d, int W, int H, int pitch, double cell_area,
                          double* partials, int max_partials, double* out, cudaStream_t st) {
  const int nb = std::max(1, std::min({H, kVolMaxBlocks, max_partials}));
  volume_rows_kernel<<<nb, kVolThreads, 0, st>>>(d, W, H, pitch, partials);
  volume_final_kernel<<<1, kVolThreads, 0, st>>>(partials, nb, cell_area, out);
  count_launch(2);
  return cudaGetLastError();
}

cudaError_t launch_generate_scene(uint64_t seed, int W, int H, int pitch, float height_scale,
                                  float fill, float* b, float* d, cudaStream_t st) {
  Lattice L{};
  long long total = 0;
  for (int o = 0; o < kOctaves; ++o) {
    const int s = 64 >> o;
    L.lx[o] = W / s + 2;
    L.n[o] = (long long)L.lx[o] * (H / s + 2);
    total += L.n[o];
    Pcg32 g;
    g.seed(seed, (uint64_t)o + 1u);
    L.base_state[o] = g.state;
    L.inc[o] = g.inc;
  }
  float* buf = nullptr;
  cudaError_t e = cudaMallocAsync(&buf, (size_t)total * sizeof(float), st);
  if (e != cudaSuccess) return e;
  long long off = 0;
  for (int o = 0; o < kOctaves; ++o) {
    L.v[o] = buf + off;
    off += L.n[o];
  }
  for (int o = 0; o < kOctaves; ++o) {
    const int nb = (int)((L.n[o] + 255) / 256);
    lattice_kernel<<<nb, 256, 0, st>>>(L, o);
  }
  dim3 blk(32, 8), grd((W + 31) / 32, (H + 7) / 8);
  scene_kernel<<<grd, blk, 0, st>>>(L, W, H, pitch, height_scale, fill, b, d);
  count_launch(kOctaves + 1);
  e = cudaGetLastError();
  cudaFreeAsync(buf, st);
  return e;
}

cudaError_t launch_flux_to_f32(const void* f, int flux_storage, float inv_scale, int W, int H,
                               int pitch, float* out_packed, cudaStream_t st) {
  dim3 blk(32, 8), grd((W + 31) / 32, (H + 7) / 8);
  flux_to_f32_kernel<<<grd, blk, 0, st>>>(f, flux_storage == TWS_FLUX_F16, inv_scale, W, H, pitch,
                                          reinterpret_cast<float4*>(out_packed));
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_flux_from_f32(const float* in_packed, int flux_storage, float scale, int W,
                                 int H, int pitch, void* f, cudaStream_t st) {
  dim3 blk(32, 8), grd((W + 31) / 32, (H + 7) / 8);
  flux_from_f32_kernel<<<grd, blk, 0, st>>>(reinterpret_cast<const float4*>(in_packed),
                                            flux_storage == TWS_FLUX_F16, scale, W, H, pitch, f);
  count_launch();
  return cudaGetLastError();
}

// ---- the reference's own noise terrain ---------------------------------------------
// Terrain::CreateHeightmapFromNoiseAndResetSim (Terrain.cpp:200-222): the
// heightmap is NoiseGenerator::GetValueNoise (NoiseGenerator.cpp:12-97) over a
// 4096-entry white-noise table drawn from the application-wide generator of
// Random.cpp (seeded once at start-up, Application.cpp:57; every generator
// takes the next 4096 numbers).  The table is made on the host (4096 numbers
// of a sequential generator), the per-cell noise on the device, in the
// reference's operation order with no contraction.
namespace {

// Random.cpp:22-57: a Mersenne-Twister-shaped state of 624 words, seeded
// with the reference's own rule.
class RefTableRng {
 public:
  explicit RefTableRng(uint32_t seed) {
    for (uint32_t k = 0; k < 624; ++k)
      st_[k] = (k & 1u) ? seed + k * 527u : (2135u + seed * 74111u) * k;
    for (int k = 0; k < 624; ++k) st_[k] = twist(st_[k], st_[(k + 1) % 624], st_[(k + 397) % 624]);
  }
  float next() {
    const int nx = (at_ + 1) % 624;
    st_[at_] = twist(st_[at_], st_[nx], st_[(at_ + 397) % 624]);
    uint32_t y = st_[at_];
    at_ = nx;
    y ^= y >> 11;
    y ^= (y << 7) & 0x9D2C5680u;
    y ^= (y << 15) & 0xEFC60000u;
    y ^= y >> 18;
    return static_cast<float>(static_cast<double>(y) * 4.656612874e-10 - 1.0);
  }

 private:
  static uint32_t twist(uint32_t lo_word, uint32_t hi_word, uint32_t far) {
    const uint32_t y = (lo_word & 0x80000000u) | (hi_word & 0x7FFFFFFFu);
    return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908B0DFu : 0u);
  }
  uint32_t st_[624];
  int at_ = 0;
};

__device__ __forceinline__ float ref_smooth(float f) {
  return fmul(fmul(fmul(f, f), f), fadd(fmul(f, fsub(fmul(f, 6.0f), 15.0f)), 10.0f));
}

// GetNoise3D for z = 0 (the terrain's only plane; the z terms keep their
// operations, with weight w = smooth(0) = 0).
__device__ float ref_noise2(const float* __restrict__ tab, float cx, float cy, int period) {
  period = period < 16 ? period : 16;
  const int mod = period - 1;
  int x0 = (int)cx, y0 = (int)cy;  // cx, cy >= 0: the reference's floor
  const float fx = fsub(cx, (float)x0), fy = fsub(cy, (float)y0);
  x0 = (x0 % period + period) & mod;
  y0 = (y0 % period + period) & mod;
  const int x1 = (x0 + 1) & mod, y1 = (y0 + 1) & mod;
  const int z1 = 1 & mod;  // z0 = 0
  const float s000 = __ldg(tab + x0 + 16 * y0), s100 = __ldg(tab + x1 + 16 * y0);
  const float s010 = __ldg(tab + x0 + 16 * y1), s110 = __ldg(tab + x1 + 16 * y1);
  const float s001 = __ldg(tab + x0 + 16 * (y0 + 16 * z1));
  const float s101 = __ldg(tab + x1 + 16 * (y0 + 16 * z1));
  const float s011 = __ldg(tab + x0 + 16 * (y1 + 16 * z1));
  const float s111 = __ldg(tab + x1 + 16 * (y1 + 16 * z1));
  const float u = ref_smooth(fx), v = ref_smooth(fy), w = ref_smooth(0.0f);
  const float uv = fmul(u, v), uw = fmul(u, w), vw = fmul(v, w);
  const float k0 = s000, k1 = fsub(s100, s000), k2 = fsub(s010, s000), k3 = fsub(s001, s000);
  const float k4 = fsub(fsub(s110, s010), k1);
  const float k5 = fadd(fsub(fsub(s000, s010), s001), s011);
  const float k6 = fadd(fsub(-k1, s001), s101);
  const float k7 = fadd(fsub(fsub(fadd(-k4, s001), s101), s011), s111);
  float r = fadd(k0, fmul(k1, u));
  r = fadd(r, fmul(k2, v));
  r = fadd(r, fmul(k3, w));
  r = fadd(r, fmul(k4, uv));
  r = fadd(r, fmul(k5, vw));
  r = fadd(r, fmul(k6, uw));
  return fadd(r, fmul(fmul(k7, uv), w));
}

__global__ void reference_scene_kernel(const float* __restrict__ tab, int W, int H, int pitch,
                                       float mx, float my, float hs, float* __restrict__ b,
                                       float* __restrict__ d) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const float cx = fmul(mx, (float)x), cy = fmul(my, (float)y);
  // GetValueNoise(octaves 2..10, persistence 0.43, periodic)
  const float persistence = 0.43f;
  float sum = 0.0f, amplitude = 1.0f, frequency = 4.0f;
  for (int octave = 2; octave <= 10; ++octave) {
    const float n = ref_noise2(tab, fmul(cx, frequency), fmul(cy, frequency), (int)frequency);
    sum = fadd(sum, fmul(amplitude, fadd(fmul(n, 0.5f), 0.5f)));
    amplitude = fmul(amplitude, persistence);
    frequency = fmul(frequency, 2.0f);
  }
  const float noise =
      fsub(fdiv(fmul(fmul(sum, 2.0f), fsub(1.0f, persistence)), fsub(1.0f, amplitude)), 1.0f);
  const float bb = fmul(fadd(fmul(noise, 0.5f), 0.5f), hs);
  const float ex = fsub(fmul((float)x, mx), 0.5f), ey = fsub(fmul((float)y, my), 0.5f);
  const float len2 = fadd(fmul(ex, ex), fmul(ey, ey));
  const float dd = fsub(fmul(fsub(0.45f, fmul(fmul(len2, len2), 800.0f)), hs), bb);
  const size_t g = (size_t)y * pitch + x;
  b[g] = bb;
  d[g] = max0(dd);
}

}  // namespace

cudaError_t launch_reference_scene(uint32_t seed, int generation, int W, int H, int pitch,
                                   float height_scale, float* b, float* d, cudaStream_t st) {
  if (W < 2 || H < 2 || generation < 0) return cudaErrorInvalidValue;
  float table[4096];
  RefTableRng rng(seed);
  for (long long i = 0; i < 4096LL * generation; ++i) rng.next();
  for (int i = 0; i < 4096; ++i) table[i] = rng.next();
  float* dtab = nullptr;
  cudaError_t e = cudaMallocAsync(&dtab, sizeof(table), st);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(dtab, table, sizeof(table), cudaMemcpyHostToDevice, st);  // staged copy
  if (e == cudaSuccess) {
    const float mx = 1.0f / (float)(W - 1), my = 1.0f / (float)(H - 1);
    dim3 blk(32, 8), grd((W + 31) / 32, (H + 7) / 8);
    reference_scene_kernel<<<grd, blk, 0, st>>>(dtab, W, H, pitch, mx, my, height_scale, b, d);
    count_launch();
    e = cudaGetLastError();
  }
  cudaFreeAsync(dtab, st);
  return e;
}

}  // namespace tws

extern "C" TWS_API int tws_scene_rain_disks(uint64_t seed, int W, int H, int radius, float rate,
                                            int count, tws_source* out) {
  if (!out || W < 1 || H < 1 || radius < 0 || count < 0 || !(rate == rate)) return TWS_ERR_INVALID;
  for (int k = 0; k < count; ++k) {
    tws::Pcg32 g;
    g.seed(seed, 1000u + (uint64_t)k);
    const uint32_t u0 = g.next(), u1 = g.next();
    const int cx = (W > 2 * radius) ? radius + (int)(u0 % (uint32_t)(W - 2 * radius)) : W / 2;
    const int cy = (H > 2 * radius) ? radius + (int)(u1 % (uint32_t)(H - 2 * radius)) : H / 2;
    out[k].kind = TWS_SOURCE_DISK;
    out[k].cx = (float)cx;
    out[k].cy = (float)cy;
    out[k].radius = (float)radius;
    out[k].rate = rate;
  }
  return TWS_OK;
}

// ---- total volume without allocation ------------------------------------------
// Scratch of tws_volume_noalloc: one FP64 partial sum per grid row, in a fixed
// array that lives in the module image, so the call needs no cudaMalloc.
// Every GPU that loads this library holds it (128 KB) until the process
// exits.  Host code must not pass `g_volume_row_sums` itself to a kernel: on
// the host that name is only a stand-in for the symbol, not a device address;
// the device address is looked up once per device below.
static __device__ __align__(256) double g_volume_row_sums[TWS_VOLUME_NOALLOC_MAX_ROWS];

namespace {

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_scratch[kNoallocMaxDevices] = {};

// Device address of the scratch on the current device; looked up on the first
// call per device (cudaGetSymbolAddress, with that device current).
cudaError_t noalloc_scratch(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kNoallocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_scratch[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_volume_row_sums);
    if (e != cudaSuccess) return e;
    g_noalloc_scratch[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_scratch[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" TWS_API int tws_volume_noalloc(const float* depth, int width, int height, int pitch,
                                          double cell_area, double* out, void* stream) {
  if (!depth || !out || width < 1 || height < 1 || pitch < width) return TWS_ERR_INVALID;
  // the kernels read floats and write a double: natural alignment
  if (reinterpret_cast<uintptr_t>(depth) % alignof(float) != 0 ||
      reinterpret_cast<uintptr_t>(out) % alignof(double) != 0)
    return TWS_ERR_INVALID;
  if (height > TWS_VOLUME_NOALLOC_MAX_ROWS) return TWS_ERR_TOO_LARGE;
  double* scratch = nullptr;
  if (noalloc_scratch(&scratch) != cudaSuccess) return TWS_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // One block per row: block r writes partial r (every partial is rewritten,
  // so nothing needs clearing); one block then adds the partials in row order.
  // Each launch's own result is checked (cudaLaunchKernelEx returns it), so
  // an earlier error pending on this thread is neither reported nor cleared.
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)height);
  cfg.blockDim = dim3(tws::kVolThreads);
  cfg.stream = st;
  cudaError_t e = cudaLaunchKernelEx(&cfg, tws::volume_rows_kernel, depth, width, height, pitch,
                                     scratch);
  if (e == cudaSuccess) {
    tws::count_launch(1);
    cfg.gridDim = dim3(1);
    e = cudaLaunchKernelEx(&cfg, tws::volume_final_kernel, static_cast<const double*>(scratch),
                           height, cell_area, out);
    if (e == cudaSuccess) tws::count_launch(1);
  }
  return e == cudaSuccess ? TWS_OK : TWS_ERR_CUDA;
}
