// tws_oracle.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// CPU restatement of terrainwatersim's virtual-pipe shallow-water step, used only
// as the correctness checker (tests/, the smoke check) and as the timed CPU
// baseline (bench.py).  The product path (libtws.so) never links, loads or calls
// this file.
//
// It follows the reference's arithmetic in the same operation order:
//   * flux update   terrainwatersim/shader/flowUpdate.comp:34-62
//   * depth / flow  terrainwatersim/shader/flowApply.comp:32-52
//   * parameters    terrainwatersim/shader/simulationCommon.glsl:1-13,
//                   terrainwatersim/source/scene/Terrain.cpp:175-198
//   * brush source  terrainwatersim/shader/waterBrush.comp:26-28 (+ helper.glsl:68)
//   * step order    terrainwatersim/source/scene/Terrain.cpp:253-265 (all fluxes,
//                   then all depths; the brush runs before the step,
//                   terrainwatersim/source/scene/Scene.cpp:354-363)
// GLSL semantics kept: an out-of-range imageLoad reads zero (boundary OPEN),
// max(x, y) = (x < y) ? y : x, left-to-right '+' chains, vec4 ops per component.
// The closed-wall boundary (zero flux across the border) is this project's
// addition for the benchmark configurations; it differs from OPEN only in the
// outflow component that points off the grid, which it forces to zero.
//
// Pinning: the FP32 OPEN-boundary path is checked bit-for-bit against the
// reference's own shader source executed on the CPU (oracle/ref_glsl, built by
// oracle/Makefile into oracle/_ref) and against the fixtures in tests/golden.
//
// Built twice from one template: float (the FP32 transcription) and double (the
// FP64 oracle).  Must be compiled with -ffp-contract=off (no FMA contraction).
//
// Also holds the synthetic scene generator (seeded PCG32 value-noise fBm) that
// the product library restates on the host and on the device; tests check the
// two agree bit for bit.

#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// Source term applied at the start of every step (before the flux update).
//   kind 0 = DISK  : every cell with (x-cx)^2 + (y-cy)^2 <= r^2 (integer cells)
//                    gains `rate` metres of water.
//   kind 1 = BRUSH : the reference's radial brush, waterBrush.comp:26-28,
//                    d += saturate(1 - |(cx,cy) - (x,y)|^2 / size_sq) * rate.
typedef struct tws_oracle_source {
  int kind;
  int pad_;
  double cx, cy;
  double radius;   // DISK: radius in cells (integer valued); BRUSH: BrushSizeSq
  double rate;     // DISK: metres per step; BRUSH: BrushIntensity
} tws_oracle_source;

}  // extern "C"

namespace {

template <class T>
struct F4 {
  T x, y, z, w;
};
template <class T>
struct F2 {
  T x, y;
};

// GLSL max(0, v): returns v if 0 < v, else 0 (flowUpdate.comp:54, flowApply.comp:41).
template <class T>
inline T glsl_max0(T v) {
  return (T(0) < v) ? v : T(0);
}

// GLSL clamp(v, 0, 1) = min(max(v, 0), 1) (helper.glsl:68 `saturate`).
template <class T>
inline T glsl_saturate(T v) {
  T m = (v < T(0)) ? T(0) : v;   // max(v, 0) = (v < 0) ? 0 : v
  return (T(1) < m) ? T(1) : m;  // min(m, 1) = (1 < m) ? 1 : m
}

template <class T>
struct Params {
  T kf;  // FlowFriction_perStep
  T ka;  // WaterAcceleration_perStep
  T c;   // CellAreaInv_timeScaled
  int closed;
  T flux_scale;  // > 0: flux is stored as IEEE half of flux * flux_scale (FP32 only)
};

// The value an FP16-stored flux reads back as: half(min(v * scale, 65504)),
// rounded to nearest even, times 1/scale (scale is a power of two).
template <class T>
inline T quantize_half(T v, T scale) {
  T s = v * scale;
  s = (s < T(65504)) ? s : T(65504);
  const _Float16 h = (_Float16)(float)s;
  return (T)((float)h) * (T(1) / scale);
}

inline int num_threads(int requested) {
#ifdef _OPENMP
  return requested > 0 ? requested : omp_get_max_threads();
#else
  (void)requested;
  return 1;
#endif
}

// The integer hash "lowbias32" (C. Wellons, hash-prospector: xorshift-multiply,
// constants 0x7feb352d and 0x846ca68b).
inline uint32_t rain_hash32(uint32_t v) {
  v ^= v >> 16;
  v *= 0x7feb352du;
  v ^= v >> 15;
  v *= 0x846ca68bu;
  v ^= v >> 16;
  return v;
}

// d + rate for the DISK rain on FP32 depths, rounded without bias.  Round to
// nearest alone biases a 0.01 m increment by a fixed fraction of an ulp of d
// (+0.24 ulp on 8-16 m, -0.44 on 32-64 m, ...), so the total volume drifts by
// up to about 2e-4 of the rain.  Here the exact rounding error e of s = d + r
// comes from TwoSum (Knuth), and s moves one ulp toward d + r when
// u * |step| < |e|, with u in [0, 1) from a hash of the cell and the bits of
// d: the expected result is d + r exactly.  Every operation is exact or
// IEEE round-to-nearest, so the GPU kernels reproduce it bit for bit.  The
// FP64 path adds plainly (its rounding is far below what is measured).
inline float add_rain(float d, float r, int x, int y) {
  const float s = d + r;
  const float bp = s - d;
  const float e = (d - (s - bp)) + (r - bp);
  if (e == 0.0f) return s;
  uint32_t sb, db;
  std::memcpy(&sb, &s, 4);
  std::memcpy(&db, &d, 4);
  sb = ((s > 0.0f) == (e > 0.0f)) ? sb + 1u : sb - 1u;  // the neighbour toward d + r
  float next;
  std::memcpy(&next, &sb, 4);
  const float step = next - s;
  const uint32_t h = rain_hash32(db ^ rain_hash32((uint32_t)x ^ rain_hash32((uint32_t)y)));
  const float u = (float)(h >> 8) * 0x1p-24f;
  return (u * std::fabs(step) < std::fabs(e)) ? next : s;
}
inline double add_rain(double d, double r, int, int) { return d + r; }

// Source term.  DISK follows the benchmark's uniform rain disk (add_rain);
// BRUSH follows waterBrush.comp:26-28: toBrush = BrushPos - gridPosition;
// q = dot / S; d += saturate(1 - q) * I.  Cells where the increment is zero
// are left as they are (d + 0 == d for every d >= +0, the only depths the
// step produces).
template <class T>
void apply_sources(int W, int H, T* d, const tws_oracle_source* src, int nsrc, int nth) {
  for (int k = 0; k < nsrc; ++k) {
    const tws_oracle_source& s = src[k];
    if (s.kind == 0) {
      const int cx = (int)s.cx, cy = (int)s.cy, r = (int)s.radius;
      const long long r2 = (long long)r * r;
      const T rate = (T)s.rate;
      const int y0 = cy - r < 0 ? 0 : cy - r, y1 = cy + r >= H ? H - 1 : cy + r;
      const int x0 = cx - r < 0 ? 0 : cx - r, x1 = cx + r >= W ? W - 1 : cx + r;
#pragma omp parallel for num_threads(nth) schedule(static)
      for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x) {
          const long long dx = x - cx, dy = y - cy;
          if (dx * dx + dy * dy <= r2)
            d[(size_t)y * W + x] = add_rain(d[(size_t)y * W + x], rate, x, y);
        }
    } else {
      const T bx = (T)s.cx, by = (T)s.cy, S = (T)s.radius, I = (T)s.rate;
#pragma omp parallel for num_threads(nth) schedule(static)
      for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
          const T tx = bx - (T)x, ty = by - (T)y;
          const T q = (tx * tx + ty * ty) / S;
          const T inc = glsl_saturate(T(1) - q) * I;
          if (inc != T(0)) d[(size_t)y * W + x] = d[(size_t)y * W + x] + inc;
        }
    }
  }
}

// flowUpdate.comp:34-62, in place on f (the shader reads and writes only its own
// cell's flux, so in-place is exact).  Channel order: x = +x, y = -x, z = +y, w = -y.
template <class T>
void flux_update(int W, int H, const Params<T>& p, const T* b, const T* d, F4<T>* f, int nth) {
#pragma omp parallel for num_threads(nth) schedule(static)
  for (int y = 0; y < H; ++y) {
    const size_t row = (size_t)y * W;
    for (int x = 0; x < W; ++x) {
      const size_t i = row + x;
      const T hc = d[i] + b[i];                                   // :34
      const T hx1 = (x + 1 < W) ? d[i + 1] + b[i + 1] : T(0);    // :37-40, OOB reads 0
      const T hx0 = (x > 0) ? d[i - 1] + b[i - 1] : T(0);
      const T hy1 = (y + 1 < H) ? d[i + W] + b[i + W] : T(0);
      const T hy0 = (y > 0) ? d[i - W] + b[i - W] : T(0);
      const T ex1 = hc - hx1, ex0 = hc - hx0, ey1 = hc - hy1, ey0 = hc - hy0;  // :44-47
      const F4<T> fo = f[i];                                                   // :50
      F4<T> nf;                                                                // :53
      nf.x = fo.x * p.kf + ex1 * p.ka;
      nf.y = fo.y * p.kf + ex0 * p.ka;
      nf.z = fo.z * p.kf + ey1 * p.ka;
      nf.w = fo.w * p.kf + ey0 * p.ka;
      nf.x = glsl_max0(nf.x);  // :54
      nf.y = glsl_max0(nf.y);
      nf.z = glsl_max0(nf.z);
      nf.w = glsl_max0(nf.w);
      if (p.closed) {  // zero flux across the outer wall
        if (x + 1 >= W) nf.x = T(0);
        if (x == 0) nf.y = T(0);
        if (y + 1 >= H) nf.z = T(0);
        if (y == 0) nf.w = T(0);
      }
      const T total = (((nf.x + nf.y) + nf.z) + nf.w) * p.c;  // :57
      const T dc = d[i];
      if (total > dc) {  // :58-59
        const T s = dc / total;
        nf.x = nf.x * s;
        nf.y = nf.y * s;
        nf.z = nf.z * s;
        nf.w = nf.w * s;
      }
      if (p.flux_scale > T(0)) {  // FP16 flux storage: the apply uses the stored value
        nf.x = quantize_half(nf.x, p.flux_scale);
        nf.y = quantize_half(nf.y, p.flux_scale);
        nf.z = quantize_half(nf.z, p.flux_scale);
        nf.w = quantize_half(nf.w, p.flux_scale);
      }
      f[i] = nf;  // :62
    }
  }
}

// flowApply.comp:32-52, in place on d (reads only its own cell's depth).
template <class T>
void flow_apply(int W, int H, const Params<T>& p, T* d, const F4<T>* f, F2<T>* v, int nth) {
#pragma omp parallel for num_threads(nth) schedule(static)
  for (int y = 0; y < H; ++y) {
    const size_t row = (size_t)y * W;
    for (int x = 0; x < W; ++x) {
      const size_t i = row + x;
      const F4<T> fo = f[i];
      const T X1 = (x + 1 < W) ? f[i + 1].y : T(0);  // :32-35, OOB reads 0
      const T X0 = (x > 0) ? f[i - 1].x : T(0);
      const T Y1 = (y + 1 < H) ? f[i + W].w : T(0);
      const T Y0 = (y > 0) ? f[i - W].z : T(0);
      const T in = ((X1 + X0) + Y1) + Y0;                // :38
      const T out = ((fo.x + fo.y) + fo.z) + fo.w;       // :39
      d[i] = glsl_max0(d[i] + (in - out) * p.c);         // :41
      if (v) {
        v[i].x = (X1 - fo.x) - (X0 - fo.y);  // :45
        v[i].y = (Y1 - fo.z) - (Y0 - fo.w);  // :46
      }
    }
  }
}

template <class T>
void run_steps(int W, int H, const Params<T>& p, const T* b, T* d, F4<T>* f, F2<T>* v,
               const tws_oracle_source* src, int nsrc, int nsteps, int nth) {
  for (int s = 0; s < nsteps; ++s) {
    apply_sources(W, H, d, src, nsrc, nth);
    flux_update(W, H, p, b, d, f, nth);
    flow_apply(W, H, p, d, f, v, nth);
  }
}

// ---------------------------------------------------------------------------
// Synthetic scene generator (the benchmark's terrain, not the reference's
// NoiseGenerator): seeded PCG32 value noise, lattice spacing 64 cells, 6
// octaves (spacing halves, amplitude halves), smoothstep-bilinear
// interpolation, normalised by the amplitude sum 1.96875 and scaled.
// PCG32 is O'Neill's XSH-RR 64/32 generator (pcg-random.org, "pcg32").

const uint64_t kPcgMult = 6364136223846793005ULL;

struct Pcg32 {
  uint64_t state, inc;
  void seed(uint64_t initstate, uint64_t initseq) {
    state = 0u;
    inc = (initseq << 1u) | 1u;
    next();
    state += initstate;
    next();
  }
  uint32_t next() {
    const uint64_t old = state;
    state = old * kPcgMult + inc;
    const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((0u - rot) & 31u));
  }
  // Jump ahead by delta steps (Brown, "Random number generation with
  // arbitrary strides", 1994): the LCG composed with itself.
  void advance(uint64_t delta) {
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

inline float u01(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }

inline float smooth01(float t) {
  const float a = t * t;
  const float c = 3.0f - 2.0f * t;
  return a * c;
}
inline float lerpf(float a, float b, float t) { return a + (b - a) * t; }

}  // namespace

extern "C" {

// Version tag of the scene generator definition; the product library reports
// the same number.
int tws_oracle_scene_version(void) { return 1; }

// Lattice value for octave o at lattice point (i, j): output number j*Lx + i of
// the PCG32 stream (seed, o + 1), mapped to [0, 1) with 24 bits.
void tws_oracle_terrain(uint64_t seed, int W, int H, float height_scale, float fill, float* b,
                        float* d) {
  const int kOct = 6;
  std::vector<std::vector<float>> lat(kOct);
  std::vector<int> lx(kOct);
  for (int o = 0; o < kOct; ++o) {
    const int s = 64 >> o;
    const int Lx = W / s + 2, Ly = H / s + 2;
    lx[o] = Lx;
    lat[o].resize((size_t)Lx * Ly);
    Pcg32 g;
    g.seed(seed, (uint64_t)o + 1u);
    for (size_t k = 0; k < lat[o].size(); ++k) lat[o][k] = u01(g.next());
  }
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      float acc = 0.0f, amp = 1.0f;
      for (int o = 0; o < kOct; ++o) {
        const int s = 64 >> o;
        const float inv = 1.0f / (float)s;
        const int i = x / s, j = y / s;
        const float sx = smooth01((float)(x % s) * inv);
        const float sy = smooth01((float)(y % s) * inv);
        const float* L = lat[o].data();
        const int Lx = lx[o];
        const float v00 = L[(size_t)j * Lx + i], v10 = L[(size_t)j * Lx + i + 1];
        const float v01 = L[(size_t)(j + 1) * Lx + i], v11 = L[(size_t)(j + 1) * Lx + i + 1];
        const float v = lerpf(lerpf(v00, v10, sx), lerpf(v01, v11, sx), sy);
        acc = acc + amp * v;
        amp = amp * 0.5f;
      }
      const float bb = (acc / 1.96875f) * height_scale;
      b[(size_t)y * W + x] = bb;
      if (d) d[(size_t)y * W + x] = glsl_max0(fill - bb);
    }
}

// Rain-disk centres: disk k draws two outputs of the PCG32 stream
// (seed, 1000 + k): cx = r + u0 % (W - 2r), cy = r + u1 % (H - 2r), so the
// disk lies inside the grid (centre of the grid if it does not fit).
void tws_oracle_rain_centers(uint64_t seed, int W, int H, int radius, int count, int* cx,
                             int* cy) {
  for (int k = 0; k < count; ++k) {
    Pcg32 g;
    g.seed(seed, 1000u + (uint64_t)k);
    const uint32_t u0 = g.next(), u1 = g.next();
    cx[k] = (W > 2 * radius) ? radius + (int)(u0 % (uint32_t)(W - 2 * radius)) : W / 2;
    cy[k] = (H > 2 * radius) ? radius + (int)(u1 % (uint32_t)(H - 2 * radius)) : H / 2;
  }
}

// Raw PCG32 outputs (for the known-answer test of the generator itself).
void tws_oracle_pcg32(uint64_t initstate, uint64_t initseq, uint64_t skip, int n, uint32_t* out) {
  Pcg32 g;
  g.seed(initstate, initseq);
  g.advance(skip);
  for (int k = 0; k < n; ++k) out[k] = g.next();
}

// Parameter derivations.
// Benchmark form: Kf = damping per step, Ka = dt*g*A/l, C = dt/l^2, evaluated in
// double (simulationCommon.glsl:8-11 states these formulas).
void tws_oracle_params_physical(double dt, double g, double A, double l, double damping,
                                double out[3]) {
  out[0] = damping;
  out[1] = dt * g * A / l;
  out[2] = dt / (l * l);
}
// Reference form, Terrain.cpp:175-198: step = 1/steps_per_second (float, held
// as double seconds), cellDistance = world/res (float);
// Kf = powf(damping, (float)step), Ka = (float)(step*accel*cellDistance),
// C = (float)(step / (cellDistance*cellDistance)).
void tws_oracle_params_reference(float steps_per_second, float damping, float accel,
                                 float world_size, unsigned resolution, float out[3]) {
  const double step = (double)(1.0f / steps_per_second);
  const float cell = world_size / (float)resolution;
  out[0] = powf(damping, (float)step);
  out[1] = (float)(step * (double)accel * (double)cell);
  out[2] = (float)(step / (double)(cell * cell));
}

// One or more steps in FP32, in place on b/d/f/v (row-major W x H; f holds 4
// floats per cell, v 2 floats per cell, v may be NULL).  Returns elapsed
// seconds of the step loop (steady clock).
// flux_scale > 0 selects FP16 flux storage with that power-of-two scale
// (the caller stores the initial flux already quantized).
double tws_oracle_step_f32(int W, int H, float kf, float ka, float c, int closed, float flux_scale,
                           const float* b, float* d, float* f, float* v,
                           const tws_oracle_source* src, int nsrc, int nsteps, int nthreads) {
  Params<float> p{kf, ka, c, closed, flux_scale};
  const int nth = num_threads(nthreads);
  const auto t0 = std::chrono::steady_clock::now();
  run_steps<float>(W, H, p, b, d, reinterpret_cast<F4<float>*>(f), reinterpret_cast<F2<float>*>(v),
                   src, nsrc, nsteps, nth);
  const auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

double tws_oracle_step_f64(int W, int H, double kf, double ka, double c, int closed,
                           const double* b, double* d, double* f, double* v,
                           const tws_oracle_source* src, int nsrc, int nsteps, int nthreads) {
  Params<double> p{kf, ka, c, closed, 0.0};
  const int nth = num_threads(nthreads);
  const auto t0 = std::chrono::steady_clock::now();
  run_steps<double>(W, H, p, b, d, reinterpret_cast<F4<double>*>(f),
                    reinterpret_cast<F2<double>*>(v), src, nsrc, nsteps, nth);
  const auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// Quantize a flux array to FP16 storage values in place (n floats).
void tws_oracle_quantize_f16(float* f, long long n, float scale) {
  for (long long i = 0; i < n; ++i) f[i] = quantize_half(f[i], scale);
}

// Only the source term (the reference's one-shot brush dispatch, Terrain.cpp:150-168).
void tws_oracle_sources_f32(int W, int H, float* d, const tws_oracle_source* src, int nsrc) {
  apply_sources<float>(W, H, d, src, nsrc, num_threads(0));
}

// Total water volume, sum of d in FP64 in row-major order, times the cell area.
double tws_oracle_volume_f32(const float* d, long long n, double cell_area) {
  double s = 0.0;
  for (long long i = 0; i < n; ++i) s += (double)d[i];
  return s * cell_area;
}
double tws_oracle_volume_f64(const double* d, long long n, double cell_area) {
  double s = 0.0;
  for (long long i = 0; i < n; ++i) s += d[i];
  return s * cell_area;
}

// ---------------------------------------------------------------------------
// What the renderer reads (the water shaders' per-texel arithmetic), on
// tightly packed W x H arrays; v holds 2 floats per cell.
//   height = d + b                                  waterRender.vert:23
//   dry = d < 0.1                                   waterRender.vert:22
//   render_height = (d + b) - 0.1, minus 10 if dry  waterRender.eval:33-35
//   normal = normalize(cross((0, h1-h0, 1), (1, h2-h3, 0))) with the four
//            neighbours wrapping around (REPEAT sampler)  waterRender.frag:50-62
//   flow = RG16F(v); speed = sqrt(dot(flow, flow));
//   foam = saturate(dot(flow, flow) * 0.00004)      waterRender.frag:240-241, 341, 346
// normalize is v / sqrt(dot(v, v)); the flow map rounds to nearest half.
void tws_oracle_surface(int W, int H, const float* b, const float* d, const float* v,
                        float* height, float* render_height, float* normal, float* speed,
                        float* foam, unsigned char* dry) {
  auto h = [&](int x, int y) { return d[(size_t)y * W + x] + b[(size_t)y * W + x]; };
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t i = (size_t)y * W + x;
      const float hc = h(x, y);
      if (height) height[i] = hc;
      if (dry) dry[i] = d[i] < 0.1f ? 1 : 0;
      if (render_height) {
        float t = hc - 0.1f;
        if (d[i] < 0.1f) t = t - 10.0f;
        render_height[i] = t;
      }
      if (normal) {
        const int xm = x == 0 ? W - 1 : x - 1, xp = x + 1 == W ? 0 : x + 1;
        const int ym = y == 0 ? H - 1 : y - 1, yp = y + 1 == H ? 0 : y + 1;
        const float A = h(x, yp) - h(x, ym), B = h(xp, y) - h(xm, y);
        // GLSL's cross(x, y) = (x1 y2 - y1 x2, x2 y0 - y2 x0, x0 y1 - y0 x1)
        // on x = (0, A, 1), y = (1, B, 0), product by product (the zero
        // products keep the sign of zero of a flat surface)
        const float nx = A * 0.0f - B * 1.0f, ny = 1.0f * 1.0f - 0.0f * 0.0f,
                    nz = 0.0f * B - 1.0f * A;
        const float len = std::sqrt((nx * nx + ny * ny) + nz * nz);
        normal[3 * i + 0] = nx / len;
        normal[3 * i + 1] = ny / len;
        normal[3 * i + 2] = nz / len;
      }
      if (speed || foam) {
        const float fx = (float)(_Float16)v[2 * i], fy = (float)(_Float16)v[2 * i + 1];
        const float s2 = fx * fx + fy * fy;
        if (speed) speed[i] = std::sqrt(s2);
        if (foam) foam[i] = glsl_saturate(s2 * 0.00004f);
      }
    }
}

// TerrainData as RGBA32F (r = b, g = b = 0.3, a = d; Terrain.cpp:216-220), then
// `levels` 2x2 box-filtered mip levels, each ((t00 + t10) + (t01 + t11)) * 0.25
// per channel, packed level after level in `mips`.
void tws_oracle_terrain_mips(int W, int H, const float* b, const float* d, int levels,
                             float* rgba, float* mips) {
  for (size_t i = 0; i < (size_t)W * H; ++i) {
    rgba[4 * i + 0] = b[i];
    rgba[4 * i + 1] = 0.3f;
    rgba[4 * i + 2] = 0.3f;
    rgba[4 * i + 3] = d[i];
  }
  const float* src = rgba;
  float* dst = mips;
  int sw = W, sh = H;
  for (int l = 1; l <= levels; ++l) {
    const int dw = sw / 2, dh = sh / 2;
    for (int y = 0; y < dh; ++y)
      for (int x = 0; x < dw; ++x)
        for (int c = 0; c < 4; ++c) {
          const float t00 = src[4 * ((size_t)(2 * y) * sw + 2 * x) + c];
          const float t10 = src[4 * ((size_t)(2 * y) * sw + 2 * x + 1) + c];
          const float t01 = src[4 * ((size_t)(2 * y + 1) * sw + 2 * x) + c];
          const float t11 = src[4 * ((size_t)(2 * y + 1) * sw + 2 * x + 1) + c];
          dst[4 * ((size_t)y * dw + x) + c] = ((t00 + t10) + (t01 + t11)) * 0.25f;
        }
    src = dst;
    dst += 4 * (size_t)dw * dh;
    sw = dw;
    sh = dh;
  }
}

int tws_oracle_max_threads(void) { return num_threads(0); }

}  // extern "C"

// ---- the reference's own noise terrain -------------------------------------------
// Terrain::CreateHeightmapFromNoiseAndResetSim (Terrain.cpp:200-222) fills the
// heightmap from NoiseGenerator::GetValueNoise (NoiseGenerator.cpp:12-40,
// GetNoise3D 42-97), whose 4096-entry white-noise table comes from the
// application-wide generator of Random.cpp (seeded once, Application.cpp:57;
// each NoiseGenerator takes the next 4096 numbers).  Restated here in the
// reference's operation order, evaluated left to right with no contraction.
namespace {

// The table generator of Random.cpp:22-57: a Mersenne-Twister-shaped state of
// 624 words with the reference's own seeding rule.
struct RefTableRng {
  uint32_t st[624];
  int at = 0;
  static uint32_t twist(uint32_t lo_word, uint32_t hi_word, uint32_t far) {
    const uint32_t y = (lo_word & 0x80000000u) | (hi_word & 0x7FFFFFFFu);
    return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908B0DFu : 0u);
  }
  explicit RefTableRng(uint32_t seed) {
    for (uint32_t k = 0; k < 624; ++k) st[k] = (k & 1u) ? seed + k * 527u : (2135u + seed * 74111u) * k;
    for (int k = 0; k < 624; ++k) st[k] = twist(st[k], st[(k + 1) % 624], st[(k + 397) % 624]);
  }
  float next() {
    const int nx = (at + 1) % 624;
    st[at] = twist(st[at], st[nx], st[(at + 397) % 624]);
    uint32_t y = st[at];
    at = nx;
    y ^= y >> 11;
    y ^= (y << 7) & 0x9D2C5680u;
    y ^= (y << 15) & 0xEFC60000u;
    y ^= y >> 18;
    return static_cast<float>(static_cast<double>(y) * 4.656612874e-10 - 1.0);
  }
};

inline float ref_smooth(float f) { return ((f * f) * f) * ((f * ((f * 6.0f) - 15.0f)) + 10.0f); }

inline int ref_floor(float a) {
  const int r = static_cast<int>(a);
  return r - static_cast<int>((a < 0.0f) && (a - static_cast<float>(r) != 0.0f));
}

// Trilinear value noise with quintic weights over a 16^3 table, period <= 16.
float ref_noise3(const float* table, float cx, float cy, float cz, int period) {
  period = period < 16 ? period : 16;
  const int mod = period - 1;
  int x0 = ref_floor(cx), y0 = ref_floor(cy), z0 = ref_floor(cz);
  const float fx = cx - static_cast<float>(x0), fy = cy - static_cast<float>(y0),
              fz = cz - static_cast<float>(z0);
  x0 = (x0 % period + period) & mod;
  y0 = (y0 % period + period) & mod;
  z0 = (z0 % period + period) & mod;
  const int x1 = (x0 + 1) & mod, y1 = (y0 + 1) & mod, z1 = (z0 + 1) & mod;
  auto at = [&](int x, int y, int z) { return table[x + 16 * (y + 16 * z)]; };
  const float s000 = at(x0, y0, z0), s100 = at(x1, y0, z0), s010 = at(x0, y1, z0),
              s110 = at(x1, y1, z0), s001 = at(x0, y0, z1), s101 = at(x1, y0, z1),
              s011 = at(x0, y1, z1), s111 = at(x1, y1, z1);
  const float u = ref_smooth(fx), v = ref_smooth(fy), w = ref_smooth(fz);
  const float uv = u * v, uw = u * w, vw = v * w;
  const float k0 = s000, k1 = s100 - s000, k2 = s010 - s000, k3 = s001 - s000;
  const float k4 = (s110 - s010) - k1;
  const float k5 = ((s000 - s010) - s001) + s011;
  const float k6 = ((-k1) - s001) + s101;
  const float k7 = ((((-k4) + s001) - s101) - s011) + s111;
  return ((((((k0 + k1 * u) + k2 * v) + k3 * w) + k4 * uv) + k5 * vw) + k6 * uw) + (k7 * uv) * w;
}

// GetValueNoise with the terrain's arguments: octaves 2..10, persistence 0.43,
// periodic, z = 0.  Result in [-1, 1].
float ref_terrain_noise(const float* table, float cx, float cy) {
  const float persistence = 0.43f;
  float sum = 0.0f, amplitude = 1.0f, frequency = static_cast<float>(1 << 2);
  for (int octave = 2; octave <= 10; ++octave) {
    const float n = ref_noise3(table, cx * frequency, cy * frequency, 0.0f * frequency,
                               static_cast<int>(frequency));
    sum = sum + amplitude * ((n * 0.5f) + 0.5f);
    amplitude = amplitude * persistence;
    frequency = frequency * 2.0f;
  }
  return (((sum * 2.0f) * (1.0f - persistence)) / (1.0f - amplitude)) - 1.0f;
}

}  // namespace

extern "C" {

// The white-noise table after the generator is seeded with `seed` and
// `generation` earlier tables were drawn.
void tws_oracle_reference_noise_table(uint32_t seed, int generation, float* out4096) {
  RefTableRng rng(seed);
  for (int g = 0; g < generation; ++g)
    for (int i = 0; i < 4096; ++i) rng.next();
  for (int i = 0; i < 4096; ++i) out4096[i] = rng.next();
}

// The reference scene on a W x H grid (the reference's own is square: W = H):
// b = (noise(x mx, y my) * 0.5 + 0.5) * hs and d = max(0, (0.45 - len2^2 * 800)
// * hs - b), len2 = (x mx - 0.5)^2 + (y my - 0.5)^2, mx = 1 / (W - 1), my =
// 1 / (H - 1).  pow(len2, 2) of the float overload is the rounded square.
void tws_oracle_reference_terrain(uint32_t seed, int generation, int W, int H, float height_scale,
                                  float* b, float* d) {
  std::vector<float> table(4096);
  tws_oracle_reference_noise_table(seed, generation, table.data());
  const float mx = 1.0f / static_cast<float>(W - 1), my = 1.0f / static_cast<float>(H - 1);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const float fxm = mx * static_cast<float>(x), fym = my * static_cast<float>(y);
      const float bb = ((ref_terrain_noise(table.data(), fxm, fym) * 0.5f) + 0.5f) * height_scale;
      const float ex = static_cast<float>(x) * mx - 0.5f, ey = static_cast<float>(y) * my - 0.5f;
      const float len2 = ex * ex + ey * ey;
      const float dd = ((0.45f - (len2 * len2) * 800.0f) * height_scale) - bb;
      b[(size_t)y * W + x] = bb;
      d[(size_t)y * W + x] = (0.0f < dd) ? dd : 0.0f;
    }
}

}  // extern "C"
