// tws_capi.cu -- the C ABI (include/tws.h): grid lifecycle, uploads,
// parameter derivation and step scheduling.  Host code only; kernels live in
// tws_step.cu and tws_aux.cu.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <map>
#include <vector>

#include "tws_internal.h"

namespace tws {

static std::atomic<uint64_t> g_launches{0};
void count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace tws

using namespace tws;

// Maps for one kernel variant; encoded on first use and cached.
struct VariantMaps {
  bool ready = false;
  CUtensorMap b, d[2], f[2];
  bool on_device = false;  // copied to the grid's descriptor block (batched kernel)
  bool fresh = false;      // copied since the last chain that used it
};

struct tws_grid {
  int W = 0, H = 0, pitch = 0;
  tws_sim_params params{};
  int flux_storage = TWS_FLUX_F32;
  float flux_scale = 1.0f;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int device = 0;
  float* b = nullptr;
  float* d[2] = {nullptr, nullptr};
  void* f[2] = {nullptr, nullptr};
  float2* v = nullptr;
  int cur = 0;
  int steps_per_launch = 0;  // 0: library's choice
  int variant = -1;          // pinned kernel variant, -1: automatic
  int resident = 0;          // > 0: the resident kernel runs the steps, on this many CTAs
  int auto_ctas = -1;        // the resident kernel's automatic cluster for this grid (-1: not asked yet)
  std::vector<VariantMaps> maps;
  tws_source src[TWS_MAX_SOURCES];
  int nsrc = 0;
  char* slab = nullptr;  // the one device allocation holding everything below
  double* vol_partials = nullptr;
  double* vol_out = nullptr;
  double vol_host[1] = {0.0};
  int* err = nullptr;     // device error word
  int* queue = nullptr;   // the sweep kernel's work queue (two ints, zero between launches)
  int err_host[1] = {0};
  CUtensorMap* desc = nullptr;  // device copies of the maps, 5 per variant (batched kernel)
  long long wait_cycles = kDefaultWaitCycles;  // SM clocks a tile-load wait may take
  int drop_loads = 0;     // test hook: tile loads arm their barrier but issue no copy
  tws_batch* batch = nullptr;  // batch this grid belongs to (its stream is the batch's)
  cudaStream_t home_stream = nullptr;
  // Asynchronous host I/O, made on first use: packed staging (upload b, d, f
  // then download d, f, v; 52 bytes per cell), a copy stream per direction,
  // and the events that hand each staging buffer between a copy stream and
  // the grid's stream.
  char* io_slab = nullptr;
  cudaStream_t io_up = nullptr, io_down = nullptr;
  cudaEvent_t up_copied = nullptr;    // host -> staging done
  cudaEvent_t up_consumed = nullptr;  // staging -> state done
  cudaEvent_t down_staged = nullptr;  // state -> staging done
  cudaEvent_t down_copied = nullptr;  // staging -> host done
  std::string last_error;
};

namespace {

int fail(tws_grid* g, int code, const std::string& msg) {
  if (g) g->last_error = msg;
  return code;
}

int cuda_fail(tws_grid* g, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return fail(g, e == cudaErrorMemoryAllocation ? TWS_ERR_OOM : TWS_ERR_CUDA, m);
}

#define TWS_CUDA(g, call, what)                  \
  do {                                           \
    cudaError_t e_ = (call);                     \
    if (e_ != cudaSuccess) return cuda_fail(g, e_, what); \
  } while (0)

size_t flux_bytes_per_cell(int storage) { return storage == TWS_FLUX_F16 ? 8 : 16; }

// The library's own stream-ordered memory pool per device.  Freed memory
// stays in the pool (release threshold: never) so that grids created after
// others were destroyed reuse it without going back to the driver.
cudaMemPool_t library_pool(int device) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  if (device < 0 || device >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[device]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[device] = p;
  }
  return pools[device];
}

bool params_ok(const tws_sim_params* p) {
  if (!p) return false;
  if (p->boundary != TWS_BOUNDARY_CLOSED && p->boundary != TWS_BOUNDARY_OPEN) return false;
  return std::isfinite(p->flow_friction_per_step) && std::isfinite(p->water_acceleration_per_step) &&
         std::isfinite(p->cell_area_inv_time_scaled) && std::isfinite(p->cell_area);
}

// Default F16 scale: a power of two that puts the largest possible outflow
// (d_max / C, reached when the scaling of flowUpdate.comp:57-59 engages) at
// about 2^13, leaving headroom for depth growth from sources.
float pick_flux_scale(float d_max, float c) {
  const double fmax = std::max(1.0, (double)d_max) / std::max(1e-12, (double)c);
  const int e = (int)std::floor(std::log2(8192.0 / fmax));
  return std::ldexp(1.0f, std::max(-24, std::min(24, e)));
}

VariantMaps* maps_for(tws_grid* g, int variant, std::string* why) {
  if ((int)g->maps.size() < step_variant_count()) g->maps.resize(step_variant_count());
  VariantMaps& m = g->maps[variant];
  if (!m.ready) {
    for (int i = 0; i < 2; ++i) {
      cudaError_t e = encode_step_maps(variant, g->flux_storage, g->W, g->H, g->pitch,
                                       i == 0 ? g->b : nullptr, g->d[i], g->f[i], &m.b, &m.d[i],
                                       &m.f[i], why);
      if (e != cudaSuccess) return nullptr;
    }
    m.ready = true;
  }
  return &m;
}

// Variants chosen by tws_autotune, per (width, height, flux storage).
struct TunedKey {
  int w, h, fs;
  bool operator<(const TunedKey& o) const {
    return w != o.w ? w < o.w : (h != o.h ? h < o.h : fs < o.fs);
  }
};
// The fastest tiled variant, and whether the resident kernel beat it.
struct Tuned {
  int variant = -1;
  bool resident = false;
};
std::mutex g_tuned_mu;
std::map<TunedKey, Tuned> g_tuned;

Tuned tuned_lookup(const tws_grid* g) {
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  auto it = g_tuned.find(TunedKey{g->W, g->H, g->flux_storage});
  return it == g_tuned.end() ? Tuned{} : it->second;
}

// Without tuning: two steps per launch (the unified-layout K = 2 tiles, the
// fastest variant measured on 4096^2), or the plain kernel where the grid is
// too small for whole interior tiles.  Results do not depend on the choice.
int default_steps_per_launch(const tws_grid* g) { return g->W >= 64 && g->H >= 64 ? 2 : 1; }

int chosen_variant(const tws_grid* g) {
  if (g->variant >= 0) return g->variant;
  if (g->steps_per_launch == 0) {
    const Tuned t = tuned_lookup(g);
    if (t.variant >= 0) return t.variant;
  }
  if (g->steps_per_launch == 0 && (long long)g->W * g->H >= kLargeGridCells) {
    const int v = step_variant_large_grid(g->flux_storage, g->W, g->H);
    if (v >= 0) return v;
  }
  const int k = g->steps_per_launch > 0 ? g->steps_per_launch : default_steps_per_launch(g);
  return step_variant_for(k, g->flux_storage);
}

// Calls shorter than this keep the tiled kernels when the resident kernel
// was chosen by the autotuner (whose trials are long calls): one resident
// launch loads and stores the whole state, which a step or two cannot repay.
constexpr int kResidentAutoMinSteps = 16;

// CTAs of the resident kernel if it runs a call of `nsteps` steps, else 0:
// it runs them if it was turned on for this grid, or if nothing is pinned,
// the autotuner chose it for this grid shape and the call is long enough.
int resident_ctas(tws_grid* g, int nsteps) {
  if (g->resident > 0) return g->resident;
  if (g->variant >= 0 || g->steps_per_launch != 0 || nsteps < kResidentAutoMinSteps ||
      !tuned_lookup(g).resident)
    return 0;
  if (g->auto_ctas < 0) {  // asked once per grid
    int ctas = 0;
    if (resident_supported(g->W, g->H, g->flux_storage, 0, &ctas) != cudaSuccess) {
      cudaGetLastError();
      ctas = 0;
    }
    g->auto_ctas = ctas;
  }
  return g->auto_ctas;
}

StepArgs make_step_args(const tws_grid* g) {
  StepArgs a{};
  a.W = g->W;
  a.H = g->H;
  a.pitch = g->pitch;
  a.kf = g->params.flow_friction_per_step;
  a.ka = g->params.water_acceleration_per_step;
  a.c = g->params.cell_area_inv_time_scaled;
  a.closed = g->params.boundary == TWS_BOUNDARY_CLOSED;
  a.nsrc = g->nsrc;
  for (int i = 0; i < g->nsrc; ++i) a.src[i] = make_dev_source(g->src[i]);
  a.v_out = g->v;
  a.flux_scale = g->flux_scale;
  a.flux_inv_scale = 1.0f / g->flux_scale;
  a.err = g->err;
  a.queue = g->queue;
  a.wait_cycles = g->wait_cycles;
  a.drop_loads = g->drop_loads;
  return a;
}

int enqueue_steps(tws_grid* g, int nsteps) {
  StepArgs a = make_step_args(g);
  if (const int ctas = resident_ctas(g, nsteps)) {
    for (int left = nsteps; left > 0;) {
      const int n = std::min(left, kResidentMaxSteps);
      const int nxt = g->cur ^ 1;
      a.d_out = g->d[nxt];
      a.f_out = g->f[nxt];
      const cudaError_t e = launch_resident(g->flux_storage, ctas, g->b, g->d[g->cur],
                                            g->f[g->cur], a, n, g->stream);
      if (e != cudaSuccess) return cuda_fail(g, e, "resident kernel launch");
      g->cur = nxt;
      left -= n;
    }
    return TWS_OK;
  }
  const int main_variant = chosen_variant(g);
  const int kmax = step_variant(main_variant).k;
  int left = nsteps;
  std::string why;
  while (left > 0) {
    const int k = std::min(kmax, left);
    // the remainder of a chain that is not a multiple of K runs shallower
    const int variant = k == kmax ? main_variant : step_variant_for(k, g->flux_storage);
    VariantMaps* m = nullptr;
    if (step_variant(variant).kind == kKindTile) {
      m = maps_for(g, variant, &why);
      if (!m) return fail(g, TWS_ERR_CUDA, why);
    }
    const int nxt = g->cur ^ 1;
    a.d_out = g->d[nxt];
    a.f_out = g->f[nxt];
    cudaError_t e = launch_step(variant, g->flux_storage, m ? &m->b : nullptr,
                                m ? &m->d[g->cur] : nullptr, m ? &m->f[g->cur] : nullptr, g->b,
                                g->d[g->cur], g->f[g->cur], a, g->stream);
    if (e != cudaSuccess) return cuda_fail(g, e, "step kernel launch");
    g->cur = nxt;
    left -= k;
  }
  return TWS_OK;
}

}  // namespace

extern "C" {

TWS_API const char* tws_version(void) { return "terrainwatersim-gb300 0.1 (sm_103a)"; }

TWS_API uint64_t tws_launch_count(void) { return g_launches.load(); }

TWS_API const char* tws_error_string(int code) {
  switch (code) {
    case TWS_OK: return "ok";
    case TWS_ERR_INVALID: return "invalid argument";
    case TWS_ERR_CUDA: return "CUDA error";
    case TWS_ERR_OOM: return "out of device memory";
    case TWS_ERR_TIMEOUT: return "device-side wait timed out";
    case TWS_ERR_UNSUPPORTED: return "unsupported option";
    case TWS_ERR_BUSY: return "admission refused";
    case TWS_ERR_TOO_LARGE:
      return "grid too large for the fixed scratch of tws_volume_noalloc "
             "(more than TWS_VOLUME_NOALLOC_MAX_ROWS rows)";
    default: return "unknown error";
  }
}

TWS_API const char* tws_last_error(tws_grid* g) { return g ? g->last_error.c_str() : "null grid"; }

TWS_API int tws_params_physical(double dt, double gravity, double pipe_area, double cell_size,
                                double damping_per_step, int boundary, tws_sim_params* out) {
  if (!out || !(dt > 0) || !(cell_size > 0) || !(pipe_area > 0) || !std::isfinite(gravity) ||
      !std::isfinite(damping_per_step))
    return TWS_ERR_INVALID;
  if (boundary != TWS_BOUNDARY_CLOSED && boundary != TWS_BOUNDARY_OPEN) return TWS_ERR_INVALID;
  out->flow_friction_per_step = (float)damping_per_step;
  out->water_acceleration_per_step = (float)(dt * gravity * pipe_area / cell_size);
  out->cell_area_inv_time_scaled = (float)(dt / (cell_size * cell_size));
  out->cell_area = (float)(cell_size * cell_size);
  out->boundary = boundary;
  return TWS_OK;
}

TWS_API int tws_params_reference(float steps_per_second, float flow_damping,
                                 float flow_acceleration, float grid_world_size,
                                 unsigned grid_resolution, int boundary, tws_sim_params* out) {
  if (!out || !(steps_per_second > 0) || grid_resolution == 0 || !(grid_world_size > 0))
    return TWS_ERR_INVALID;
  if (boundary != TWS_BOUNDARY_CLOSED && boundary != TWS_BOUNDARY_OPEN) return TWS_ERR_INVALID;
  // Terrain.cpp:177 -- the step length is a float 1/steps held as double seconds.
  const double step = (double)(1.0f / steps_per_second);
  // Terrain.cpp:183, 196
  const float cell = grid_world_size / (float)grid_resolution;
  out->flow_friction_per_step = powf(flow_damping, (float)step);                      // :190
  out->water_acceleration_per_step = (float)(step * (double)flow_acceleration * (double)cell);  // :197
  out->cell_area_inv_time_scaled = (float)(step / (double)(cell * cell));            // :184
  out->cell_area = cell * cell;
  out->boundary = boundary;
  return TWS_OK;
}

TWS_API int tws_create(int width, int height, const tws_sim_params* params, int flux_storage,
                       void* stream, tws_grid** out) {
  if (!out) return TWS_ERR_INVALID;
  *out = nullptr;
  // (height <= 2^19 keeps the tile rows of a one-CTA-per-tile launch within
  // the 65535 limit of a grid's y dimension for 16-row tiles)
  if (width < 1 || height < 1 || width > (1 << 20) || height > (1 << 19) || !params_ok(params))
    return TWS_ERR_INVALID;
  if (flux_storage != TWS_FLUX_F32 && flux_storage != TWS_FLUX_F16) return TWS_ERR_INVALID;
  tws_grid* g = new (std::nothrow) tws_grid();
  if (!g) return TWS_ERR_OOM;
  g->W = width;
  g->H = height;
  g->pitch = (width + 31) / 32 * 32;
  g->params = *params;
  g->flux_storage = flux_storage;
  g->flux_scale = flux_storage == TWS_FLUX_F16
                      ? pick_flux_scale(32.0f, params->cell_area_inv_time_scaled)
                      : 1.0f;
  auto bail = [&](int code) {
    tws_destroy(g);
    return code;
  };
  cudaError_t e = cudaGetDevice(&g->device);
  if (e != cudaSuccess) return bail(TWS_ERR_CUDA);
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, g->device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, g->device);
  if (major != 10 || minor != 3) {
    // The kernels are built for sm_103a only.
    return bail(TWS_ERR_CUDA);
  }
  if (stream) {
    g->stream = static_cast<cudaStream_t>(stream);
  } else {
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess)
      return bail(TWS_ERR_CUDA);
    g->own_stream = true;
  }
  const size_t n = (size_t)g->pitch * g->H;
  const size_t fb = flux_bytes_per_cell(flux_storage);
  // All device state in one stream-ordered allocation from the library's
  // pool: creating and destroying grids (the serving loop does it per
  // request) never synchronises the device.
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  const size_t ob = take(n * 4), od0 = take(n * 4), od1 = take(n * 4), of0 = take(n * fb),
               of1 = take(n * fb), ov = take(n * 8),
               op = take(sizeof(double) * volume_partials_needed()), oo = take(sizeof(double)),
               oe = take(64), ot = take(sizeof(CUtensorMap) * 5 * step_variant_count());
  cudaMemPool_t pool = library_pool(g->device);
  if (!pool || cudaMallocFromPoolAsync(reinterpret_cast<void**>(&g->slab), off, pool, g->stream) !=
                   cudaSuccess) {
    cudaGetLastError();
    return bail(TWS_ERR_OOM);
  }
  g->b = reinterpret_cast<float*>(g->slab + ob);
  g->d[0] = reinterpret_cast<float*>(g->slab + od0);
  g->d[1] = reinterpret_cast<float*>(g->slab + od1);
  g->f[0] = g->slab + of0;
  g->f[1] = g->slab + of1;
  g->v = reinterpret_cast<float2*>(g->slab + ov);
  g->vol_partials = reinterpret_cast<double*>(g->slab + op);
  g->vol_out = reinterpret_cast<double*>(g->slab + oo);
  g->err = reinterpret_cast<int*>(g->slab + oe);
  g->queue = reinterpret_cast<int*>(g->slab + oe + 16);
  g->desc = reinterpret_cast<CUtensorMap*>(g->slab + ot);
  // Zero everything, padding included (the F16 flux map reads the padding
  // cell of odd-width rows and relies on it staying zero).
  cudaMemsetAsync(g->b, 0, n * 4, g->stream);
  cudaMemsetAsync(g->d[0], 0, n * 4, g->stream);
  cudaMemsetAsync(g->d[1], 0, n * 4, g->stream);
  cudaMemsetAsync(g->f[0], 0, n * fb, g->stream);
  cudaMemsetAsync(g->f[1], 0, n * fb, g->stream);
  cudaMemsetAsync(g->v, 0, n * 8, g->stream);
  cudaMemsetAsync(g->err, 0, 64, g->stream);  // the error word and the sweep queue
  if (cudaStreamSynchronize(g->stream) != cudaSuccess) return bail(TWS_ERR_CUDA);
  *out = g;
  return TWS_OK;
}

TWS_API int tws_destroy(tws_grid* g) {
  if (!g) return TWS_ERR_INVALID;
  if (g->batch) tws_batch_remove(g->batch, g);
  // the copy streams may still read or write caller arrays: let them finish
  if (g->io_up) cudaStreamSynchronize(g->io_up);
  if (g->io_down) cudaStreamSynchronize(g->io_down);
  // stream-ordered: the memory returns to the pool once the grid's queued
  // work is done, without waiting here
  if (g->io_slab) cudaFreeAsync(g->io_slab, g->stream);
  for (cudaEvent_t ev : {g->up_copied, g->up_consumed, g->down_staged, g->down_copied})
    if (ev) cudaEventDestroy(ev);
  if (g->io_up) cudaStreamDestroy(g->io_up);
  if (g->io_down) cudaStreamDestroy(g->io_down);
  if (g->slab) cudaFreeAsync(g->slab, g->stream);
  if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
  delete g;
  return TWS_OK;
}

TWS_API void* tws_stream(tws_grid* g) { return g ? (void*)g->stream : nullptr; }

static int upload_impl(tws_grid* g, const float* b, const float* d, const float* f,
                       cudaMemcpyKind kind) {
  if (!g || !b) return fail(g, TWS_ERR_INVALID, "terrain array is required");
  const size_t row = (size_t)g->W * 4, pitch = (size_t)g->pitch * 4;
  const size_t n = (size_t)g->pitch * g->H;
  g->cur = 0;
  TWS_CUDA(g, cudaMemcpy2DAsync(g->b, pitch, b, row, row, g->H, kind, g->stream), "upload terrain");
  if (d)
    TWS_CUDA(g, cudaMemcpy2DAsync(g->d[0], pitch, d, row, row, g->H, kind, g->stream), "upload depth");
  else
    TWS_CUDA(g, cudaMemsetAsync(g->d[0], 0, n * 4, g->stream), "clear depth");
  const size_t fb = flux_bytes_per_cell(g->flux_storage);
  if (f) {
    if (g->flux_storage == TWS_FLUX_F32) {
      TWS_CUDA(g, cudaMemcpy2DAsync(g->f[0], (size_t)g->pitch * 16, f, (size_t)g->W * 16,
                                    (size_t)g->W * 16, g->H, kind, g->stream),
               "upload flux");
    } else {
      float* tmp = nullptr;
      TWS_CUDA(g, cudaMallocAsync(&tmp, (size_t)g->W * g->H * 16, g->stream), "flux staging");
      cudaMemcpyAsync(tmp, f, (size_t)g->W * g->H * 16, kind, g->stream);
      launch_flux_from_f32(tmp, g->flux_storage, g->flux_scale, g->W, g->H, g->pitch, g->f[0],
                           g->stream);
      cudaFreeAsync(tmp, g->stream);
    }
  } else {
    TWS_CUDA(g, cudaMemsetAsync(g->f[0], 0, n * fb, g->stream), "clear flux");
  }
  TWS_CUDA(g, cudaMemsetAsync(g->v, 0, n * 8, g->stream), "clear velocity");
  TWS_CUDA(g, cudaStreamSynchronize(g->stream), "upload");
  return TWS_OK;
}

TWS_API int tws_upload(tws_grid* g, const float* b, const float* d, const float* f) {
  return upload_impl(g, b, d, f, cudaMemcpyHostToDevice);
}

TWS_API int tws_upload_device(tws_grid* g, const float* b, const float* d, const float* f) {
  return upload_impl(g, b, d, f, cudaMemcpyDeviceToDevice);
}

TWS_API int tws_generate_scene(tws_grid* g, uint64_t seed, float height_scale, float fill) {
  if (!g || !(height_scale >= 0) || !std::isfinite(fill)) return fail(g, TWS_ERR_INVALID, "bad scene");
  const size_t n = (size_t)g->pitch * g->H;
  g->cur = 0;
  TWS_CUDA(g, launch_generate_scene(seed, g->W, g->H, g->pitch, height_scale, fill, g->b, g->d[0],
                                    g->stream),
           "scene generator");
  TWS_CUDA(g, cudaMemsetAsync(g->f[0], 0, n * flux_bytes_per_cell(g->flux_storage), g->stream),
           "clear flux");
  TWS_CUDA(g, cudaMemsetAsync(g->v, 0, n * 8, g->stream), "clear velocity");
  return TWS_OK;
}

TWS_API int tws_generate_reference_scene(tws_grid* g, uint32_t seed, int generation,
                                         float height_scale) {
  if (!g || generation < 0 || generation > 4096 || !(height_scale >= 0) ||
      !std::isfinite(height_scale))
    return fail(g, TWS_ERR_INVALID, "bad reference scene");
  if (g->W < 2 || g->H < 2) return fail(g, TWS_ERR_INVALID, "the reference scene needs 2x2 cells");
  const size_t n = (size_t)g->pitch * g->H;
  g->cur = 0;
  TWS_CUDA(g, launch_reference_scene(seed, generation, g->W, g->H, g->pitch, height_scale, g->b,
                                     g->d[0], g->stream),
           "reference scene");
  TWS_CUDA(g, cudaMemsetAsync(g->f[0], 0, n * flux_bytes_per_cell(g->flux_storage), g->stream),
           "clear flux");
  TWS_CUDA(g, cudaMemsetAsync(g->v, 0, n * 8, g->stream), "clear velocity");
  return TWS_OK;
}

TWS_API int tws_set_params(tws_grid* g, const tws_sim_params* p) {
  if (!g || !params_ok(p)) return fail(g, TWS_ERR_INVALID, "bad parameters");
  g->params = *p;
  return TWS_OK;
}

TWS_API int tws_set_sources(tws_grid* g, const tws_source* s, int n) {
  if (!g || n < 0 || n > TWS_MAX_SOURCES || (n > 0 && !s))
    return fail(g, TWS_ERR_INVALID, "bad source list");
  for (int i = 0; i < n; ++i) {
    if (s[i].kind != TWS_SOURCE_DISK && s[i].kind != TWS_SOURCE_BRUSH)
      return fail(g, TWS_ERR_INVALID, "bad source kind");
    if (!std::isfinite(s[i].cx) || !std::isfinite(s[i].cy) || !std::isfinite(s[i].rate) ||
        !(s[i].radius >= 0) || !std::isfinite(s[i].radius))
      return fail(g, TWS_ERR_INVALID, "non-finite source");
    if (s[i].kind == TWS_SOURCE_BRUSH && !(s[i].radius > 0))
      return fail(g, TWS_ERR_INVALID, "brush size must be positive");
    if (std::fabs(s[i].cx) > 1e8f || std::fabs(s[i].cy) > 1e8f || s[i].radius > 1e8f)
      return fail(g, TWS_ERR_INVALID, "source out of range");
  }
  for (int i = 0; i < n; ++i) g->src[i] = s[i];
  g->nsrc = n;
  return TWS_OK;
}

TWS_API int tws_apply_source(tws_grid* g, const tws_source* s) {
  if (!g || !s) return fail(g, TWS_ERR_INVALID, "null source");
  if (s->kind != TWS_SOURCE_DISK && s->kind != TWS_SOURCE_BRUSH) return fail(g, TWS_ERR_INVALID, "bad source kind");
  if (!std::isfinite(s->cx) || !std::isfinite(s->cy) || !std::isfinite(s->rate) ||
      !(s->radius >= 0) || std::fabs(s->cx) > 1e8f || std::fabs(s->cy) > 1e8f || s->radius > 1e8f)
    return fail(g, TWS_ERR_INVALID, "bad source");
  if (s->kind == TWS_SOURCE_BRUSH && !(s->radius > 0)) return fail(g, TWS_ERR_INVALID, "brush size must be positive");
  TWS_CUDA(g, launch_apply_source(g->d[g->cur], g->W, g->H, g->pitch, make_dev_source(*s), g->stream),
           "source kernel");
  return TWS_OK;
}

TWS_API int tws_set_steps_per_launch(tws_grid* g, int k) {
  if (!g || k < 0 || k > 4) return fail(g, TWS_ERR_INVALID, "steps per launch must be 0..4");
  g->steps_per_launch = k;
  g->variant = -1;
  g->resident = 0;
  return TWS_OK;
}

TWS_API int tws_resident_fits(int width, int height, int flux_storage) {
  if (flux_storage != TWS_FLUX_F32 && flux_storage != TWS_FLUX_F16) return 0;
  int ctas = 0;
  if (resident_supported(width, height, flux_storage, 0, &ctas) == cudaSuccess) return ctas;
  cudaGetLastError();
  return 0;
}

TWS_API int tws_set_resident(tws_grid* g, int ctas) {
  if (!g) return TWS_ERR_INVALID;
  if (ctas < TWS_RESIDENT_AUTO || ctas > 16) return fail(g, TWS_ERR_INVALID, "bad cluster size");
  int chosen = 0;
  if (ctas != 0) {
    const cudaError_t e = resident_supported(g->W, g->H, g->flux_storage,
                                             ctas == TWS_RESIDENT_AUTO ? 0 : ctas, &chosen);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(g, TWS_ERR_UNSUPPORTED,
                  std::string("the grid does not fit the resident kernel with this cluster: ") +
                      cudaGetErrorString(e));
    }
  }
  g->resident = chosen;
  return TWS_OK;
}

TWS_API int tws_variant_count(void) { return step_variant_count(); }

TWS_API int tws_variant_info(int i, int* k, int* tx, int* ty, int* stages, size_t* smem) {
  if (i < 0 || i >= step_variant_count()) return TWS_ERR_INVALID;
  const StepVariant& v = step_variant(i);
  if (k) *k = v.k;
  if (tx) *tx = v.tx;
  if (ty) *ty = v.ty;
  if (stages) *stages = v.stages;
  if (smem) *smem = v.smem;
  return TWS_OK;
}

TWS_API int tws_current_variant(tws_grid* g, int* variant) {
  if (!g || !variant) return TWS_ERR_INVALID;
  *variant = chosen_variant(g);
  return TWS_OK;
}

TWS_API int tws_variant_tail_rows(int i) {
  if (i < 0 || i >= step_variant_count()) return TWS_ERR_INVALID;
  return step_variant(i).kind == kKindSweep ? step_variant(i).ry_tail : 0;
}

TWS_API int tws_variant_kind(int i) {
  if (i < 0 || i >= step_variant_count()) return TWS_ERR_INVALID;
  switch (step_variant(i).kind) {
    case kKindStream: return TWS_VARIANT_STREAM;
    case kKindSweep: return TWS_VARIANT_SWEEP;
    default: return TWS_VARIANT_TILE;
  }
}

TWS_API int tws_set_variant(tws_grid* g, int variant) {
  if (!g || variant < -1 || variant >= step_variant_count())
    return fail(g, TWS_ERR_INVALID, "no such kernel variant");
  g->variant = variant;
  g->resident = 0;
  return TWS_OK;
}

TWS_API int tws_set_wait_limit(tws_grid* g, long long sm_cycles) {
  if (!g || sm_cycles < 0) return fail(g, TWS_ERR_INVALID, "wait limit must be >= 0");
  g->wait_cycles = sm_cycles == 0 ? kDefaultWaitCycles : sm_cycles;
  return TWS_OK;
}

TWS_API int tws_test_drop_tile_loads(tws_grid* g, int drop) {
  if (!g || (drop != 0 && drop != 1)) return fail(g, TWS_ERR_INVALID, "drop must be 0 or 1");
  g->drop_loads = drop;
  return TWS_OK;
}

TWS_API int tws_autotune(tws_grid* g, int trial_steps, int* chosen) {
  if (!g || trial_steps < 1) return fail(g, TWS_ERR_INVALID, "trial_steps must be positive");
  const size_t cells = (size_t)g->pitch * g->H;
  const size_t fb = flux_bytes_per_cell(g->flux_storage);
  const int steps = (trial_steps + 11) / 12 * 12;  // a multiple of every K
  // one allocation for the saved state: depth, flux, flow map
  char* saved = nullptr;
  TWS_CUDA(g, cudaMallocAsync(reinterpret_cast<void**>(&saved), cells * (4 + fb + 8), g->stream),
           "autotune state copy");
  float* sd = reinterpret_cast<float*>(saved);
  void* sf = saved + cells * 4;
  float2* sv = reinterpret_cast<float2*>(saved + cells * (4 + fb));
  const int cur0 = g->cur;
  cudaMemcpyAsync(sd, g->d[cur0], cells * 4, cudaMemcpyDeviceToDevice, g->stream);
  cudaMemcpyAsync(sf, g->f[cur0], cells * fb, cudaMemcpyDeviceToDevice, g->stream);
  cudaMemcpyAsync(sv, g->v, cells * 8, cudaMemcpyDeviceToDevice, g->stream);
  auto restore = [&]() {
    g->cur = cur0;
    cudaMemcpyAsync(g->d[cur0], sd, cells * 4, cudaMemcpyDeviceToDevice, g->stream);
    cudaMemcpyAsync(g->f[cur0], sf, cells * fb, cudaMemcpyDeviceToDevice, g->stream);
    cudaMemcpyAsync(g->v, sv, cells * 8, cudaMemcpyDeviceToDevice, g->stream);
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int saved_variant = g->variant, saved_resident = g->resident;
  g->resident = 0;
  float best_ms = 1e30f;
  int best = -1, rc = TWS_OK;
  for (int v = 0; v < step_variant_count() && rc == TWS_OK; ++v) {
    float vbest = 1e30f;
    for (int rep = 0; rep < 2 && rc == TWS_OK; ++rep) {
      restore();
      g->variant = v;
      cudaEventRecord(e0, g->stream);
      rc = enqueue_steps(g, steps);
      cudaEventRecord(e1, g->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = TWS_ERR_CUDA;
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      vbest = std::min(vbest, ms);
    }
    if (vbest < best_ms) {
      best_ms = vbest;
      best = v;
    }
  }
  // the resident kernel, where the grid fits it
  bool resident_best = false;
  int res_ctas = 0;
  if (rc == TWS_OK &&
      resident_supported(g->W, g->H, g->flux_storage, 0, &res_ctas) == cudaSuccess) {
    g->resident = res_ctas;
    float rbest = 1e30f;
    for (int rep = 0; rep < 2 && rc == TWS_OK; ++rep) {
      restore();
      cudaEventRecord(e0, g->stream);
      rc = enqueue_steps(g, steps);
      cudaEventRecord(e1, g->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = TWS_ERR_CUDA;
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      rbest = std::min(rbest, ms);
    }
    resident_best = rc == TWS_OK && rbest < best_ms;
    g->resident = 0;
  }
  cudaGetLastError();  // a grid that does not fit leaves the query's error behind
  restore();
  cudaFreeAsync(saved, g->stream);
  cudaStreamSynchronize(g->stream);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != TWS_OK) {
    g->variant = saved_variant;
    g->resident = saved_resident;
    return rc;
  }
  // a resident choice is not pinned: it runs the long calls, the fastest
  // tiled variant the short ones
  g->variant = resident_best ? -1 : best;
  g->resident = 0;
  const int choice = resident_best ? TWS_VARIANT_RESIDENT : best;
  {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    g_tuned[TunedKey{g->W, g->H, g->flux_storage}] = Tuned{best, resident_best};
  }
  if (chosen) *chosen = choice;
  return TWS_OK;
}

TWS_API int tws_step(tws_grid* g, int nsteps) {
  if (!g || nsteps < 0) return fail(g, TWS_ERR_INVALID, "bad step count");
  if (nsteps == 0) return TWS_OK;
  return enqueue_steps(g, nsteps);
}

TWS_API int tws_volume(tws_grid* g, double* out) {
  if (!g || !out) return fail(g, TWS_ERR_INVALID, "null output");
  TWS_CUDA(g, launch_volume(g->d[g->cur], g->W, g->H, g->pitch, (double)g->params.cell_area,
                            g->vol_partials, volume_partials_needed(), g->vol_out, g->stream),
           "volume kernels");
  TWS_CUDA(g, cudaMemcpyAsync(g->vol_host, g->vol_out, sizeof(double), cudaMemcpyDeviceToHost, g->stream),
           "volume copy");
  TWS_CUDA(g, cudaStreamSynchronize(g->stream), "volume");
  *out = *g->vol_host;
  return TWS_OK;
}

TWS_API int tws_download(tws_grid* g, float* d, float* f, float* v) {
  if (!g) return TWS_ERR_INVALID;
  const size_t row = (size_t)g->W * 4, pitch = (size_t)g->pitch * 4;
  if (d)
    TWS_CUDA(g, cudaMemcpy2DAsync(d, row, g->d[g->cur], pitch, row, g->H, cudaMemcpyDeviceToHost, g->stream),
             "download depth");
  if (f) {
    if (g->flux_storage == TWS_FLUX_F32) {
      TWS_CUDA(g, cudaMemcpy2DAsync(f, (size_t)g->W * 16, g->f[g->cur], (size_t)g->pitch * 16,
                                    (size_t)g->W * 16, g->H, cudaMemcpyDeviceToHost, g->stream),
               "download flux");
    } else {
      float* tmp = nullptr;
      TWS_CUDA(g, cudaMallocAsync(&tmp, (size_t)g->W * g->H * 16, g->stream), "flux staging");
      launch_flux_to_f32(g->f[g->cur], g->flux_storage, 1.0f / g->flux_scale, g->W, g->H, g->pitch, tmp,
                         g->stream);
      cudaMemcpyAsync(f, tmp, (size_t)g->W * g->H * 16, cudaMemcpyDeviceToHost, g->stream);
      cudaFreeAsync(tmp, g->stream);
    }
  }
  if (v)
    TWS_CUDA(g, cudaMemcpy2DAsync(v, (size_t)g->W * 8, g->v, (size_t)g->pitch * 8, (size_t)g->W * 8,
                                  g->H, cudaMemcpyDeviceToHost, g->stream),
             "download velocity");
  TWS_CUDA(g, cudaStreamSynchronize(g->stream), "download");
  return TWS_OK;
}

TWS_API int tws_download_terrain(tws_grid* g, float* b) {
  if (!g || !b) return TWS_ERR_INVALID;
  const size_t row = (size_t)g->W * 4, pitch = (size_t)g->pitch * 4;
  TWS_CUDA(g, cudaMemcpy2DAsync(b, row, g->b, pitch, row, g->H, cudaMemcpyDeviceToHost, g->stream),
           "download terrain");
  TWS_CUDA(g, cudaStreamSynchronize(g->stream), "download terrain");
  return TWS_OK;
}

}  // extern "C"

namespace {

// Staging of the asynchronous host I/O: W x H packed arrays, each starting
// on a 256-byte boundary (the flux conversions move float4s), upload side
// (b, d, f as 4 floats) then download side (d, f as 4 floats, v as 2).
struct IoStaging {
  float *up_b, *up_d, *up_f, *down_d, *down_f, *down_v;
};

// Byte offsets of the six arrays for W x H = m cells; returns the total.
size_t io_layout(size_t m, size_t off[6]) {
  const size_t floats[6] = {m, m, 4 * m, m, 4 * m, 2 * m};
  size_t o = 0;
  for (int i = 0; i < 6; ++i) {
    off[i] = o;
    o += (floats[i] * 4 + 255) / 256 * 256;
  }
  return o;
}

IoStaging io_staging(const tws_grid* g) {
  size_t off[6];
  io_layout((size_t)g->W * g->H, off);
  float* a[6];
  for (int i = 0; i < 6; ++i) a[i] = reinterpret_cast<float*>(g->io_slab + off[i]);
  return {a[0], a[1], a[2], a[3], a[4], a[5]};
}

// All or nothing: the grid has the staging, both copy streams and the four
// events, or none of them.
int ensure_io(tws_grid* g) {
  if (g->io_slab) return TWS_OK;
  cudaStream_t up = nullptr, down = nullptr;
  cudaEvent_t ev[4] = {};
  char* slab = nullptr;
  bool ok = cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking) == cudaSuccess;
  for (int i = 0; ok && i < 4; ++i)
    ok = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) == cudaSuccess;
  cudaMemPool_t pool = ok ? library_pool(g->device) : nullptr;
  size_t off[6];
  const size_t bytes = io_layout((size_t)g->W * g->H, off);
  ok = ok && pool &&
       cudaMallocFromPoolAsync(reinterpret_cast<void**>(&slab), bytes, pool, g->stream) ==
           cudaSuccess;
  // the copy streams touch the staging only once its allocation has happened
  ok = ok && cudaStreamSynchronize(g->stream) == cudaSuccess;
  if (!ok) {
    const cudaError_t e = cudaGetLastError();
    if (slab) cudaFreeAsync(slab, g->stream);
    for (cudaEvent_t x : ev)
      if (x) cudaEventDestroy(x);
    if (up) cudaStreamDestroy(up);
    if (down) cudaStreamDestroy(down);
    return cuda_fail(g, e == cudaSuccess ? cudaErrorMemoryAllocation : e, "host I/O staging");
  }
  g->io_slab = slab;
  g->io_up = up;
  g->io_down = down;
  g->up_copied = ev[0];
  g->up_consumed = ev[1];
  g->down_staged = ev[2];
  g->down_copied = ev[3];
  return TWS_OK;
}

}  // namespace

extern "C" {

TWS_API int tws_upload_async(tws_grid* g, const float* b, const float* d, const float* f) {
  if (!g || !b) return fail(g, TWS_ERR_INVALID, "terrain array is required");
  if (const int rc = ensure_io(g)) return rc;
  const IoStaging s = io_staging(g);
  const size_t m = (size_t)g->W * g->H, n = (size_t)g->pitch * g->H;
  // host -> staging on the upload stream, once the previous upload has left
  // the staging
  TWS_CUDA(g, cudaStreamWaitEvent(g->io_up, g->up_consumed, 0), "upload order");
  TWS_CUDA(g, cudaMemcpyAsync(s.up_b, b, m * 4, cudaMemcpyHostToDevice, g->io_up), "upload terrain");
  if (d)
    TWS_CUDA(g, cudaMemcpyAsync(s.up_d, d, m * 4, cudaMemcpyHostToDevice, g->io_up), "upload depth");
  if (f)
    TWS_CUDA(g, cudaMemcpyAsync(s.up_f, f, m * 16, cudaMemcpyHostToDevice, g->io_up), "upload flux");
  TWS_CUDA(g, cudaEventRecord(g->up_copied, g->io_up), "upload order");
  // staging -> state in the grid's stream order: one copy launch on the SMs
  // (terrain, depth, FP32 flux, the cleared flow map)
  TWS_CUDA(g, cudaStreamWaitEvent(g->stream, g->up_copied, 0), "upload order");
  g->cur = 0;
  const int P = g->pitch, W = g->W;
  StageRows sr{};
  sr.add(s.up_b, W, g->b, P, W);
  if (d)
    sr.add(s.up_d, W, g->d[0], P, W);
  else
    sr.add(nullptr, P, g->d[0], P, P);
  const bool f32 = g->flux_storage == TWS_FLUX_F32;
  if (f32)
    sr.add(f ? s.up_f : nullptr, f ? 4 * W : 4 * P, reinterpret_cast<float*>(g->f[0]), 4 * P,
           f ? 4 * W : 4 * P);
  sr.add(nullptr, 2 * P, reinterpret_cast<float*>(g->v), 2 * P, 2 * P);
  TWS_CUDA(g, launch_stage_rows(sr, g->H, g->stream), "stage state");
  if (!f32 && f)
    TWS_CUDA(g, launch_flux_from_f32(s.up_f, g->flux_storage, g->flux_scale, g->W, g->H, g->pitch,
                                     g->f[0], g->stream),
             "stage flux");
  else if (!f32)
    TWS_CUDA(g, cudaMemsetAsync(g->f[0], 0, n * flux_bytes_per_cell(g->flux_storage), g->stream),
             "clear flux");
  TWS_CUDA(g, cudaEventRecord(g->up_consumed, g->stream), "upload order");
  return TWS_OK;
}

TWS_API int tws_download_async(tws_grid* g, float* d, float* f, float* v) {
  if (!g) return TWS_ERR_INVALID;
  if (const int rc = ensure_io(g)) return rc;
  const IoStaging s = io_staging(g);
  const size_t m = (size_t)g->W * g->H;
  // state -> staging in the grid's stream order, once the previous download
  // has left the staging
  TWS_CUDA(g, cudaStreamWaitEvent(g->stream, g->down_copied, 0), "download order");
  const int P = g->pitch, W = g->W;
  const bool f32 = g->flux_storage == TWS_FLUX_F32;
  StageRows sr{};
  if (d) sr.add(g->d[g->cur], P, s.down_d, W, W);
  if (f && f32)
    sr.add(reinterpret_cast<const float*>(g->f[g->cur]), 4 * P, s.down_f, 4 * W, 4 * W);
  if (v) sr.add(reinterpret_cast<const float*>(g->v), 2 * P, s.down_v, 2 * W, 2 * W);
  TWS_CUDA(g, launch_stage_rows(sr, g->H, g->stream), "stage state");
  if (f && !f32)
    TWS_CUDA(g, launch_flux_to_f32(g->f[g->cur], g->flux_storage, 1.0f / g->flux_scale, g->W, g->H,
                                   g->pitch, s.down_f, g->stream),
             "stage flux");
  TWS_CUDA(g, cudaEventRecord(g->down_staged, g->stream), "download order");
  // staging -> host on the download stream
  TWS_CUDA(g, cudaStreamWaitEvent(g->io_down, g->down_staged, 0), "download order");
  if (d)
    TWS_CUDA(g, cudaMemcpyAsync(d, s.down_d, m * 4, cudaMemcpyDeviceToHost, g->io_down),
             "download depth");
  if (f)
    TWS_CUDA(g, cudaMemcpyAsync(f, s.down_f, m * 16, cudaMemcpyDeviceToHost, g->io_down),
             "download flux");
  if (v)
    TWS_CUDA(g, cudaMemcpyAsync(v, s.down_v, m * 8, cudaMemcpyDeviceToHost, g->io_down),
             "download velocity");
  TWS_CUDA(g, cudaEventRecord(g->down_copied, g->io_down), "download order");
  return TWS_OK;
}

TWS_API int tws_io_wait(tws_grid* g) {
  if (!g) return TWS_ERR_INVALID;
  if (g->io_up) TWS_CUDA(g, cudaStreamSynchronize(g->io_up), "upload");
  if (g->io_down) TWS_CUDA(g, cudaStreamSynchronize(g->io_down), "download");
  return TWS_OK;
}

TWS_API int tws_surface(tws_grid* g, const tws_surface_out* o) {
  if (!g || !o) return fail(g, TWS_ERR_INVALID, "null surface output");
  // the float outputs are written as floats at least: natural alignment
  for (const void* p : {(const void*)o->height, (const void*)o->render_height,
                        (const void*)o->normal, (const void*)o->flow_speed, (const void*)o->foam})
    if (reinterpret_cast<uintptr_t>(p) % 4 != 0)
      return fail(g, TWS_ERR_INVALID, "surface outputs must be 4-byte aligned");
  TWS_CUDA(g, launch_surface(g->b, g->d[g->cur], g->v, g->W, g->H, g->pitch, *o, g->stream),
           "surface kernel");
  return TWS_OK;
}

TWS_API int tws_export_textures(tws_grid* g, float* terrain_rgba, uint16_t* flowmap,
                                int mip_levels, float* mips) {
  if (!g || mip_levels < 0) return fail(g, TWS_ERR_INVALID, "bad export arguments");
  if (mip_levels > 0 && (!terrain_rgba || !mips))
    return fail(g, TWS_ERR_INVALID, "mips need terrain_rgba and mips buffers");
  // RGBA32F texels are moved as 16-byte vectors, RG16F texels as 4-byte pairs
  if (reinterpret_cast<uintptr_t>(terrain_rgba) % 16 != 0 ||
      reinterpret_cast<uintptr_t>(mips) % 16 != 0)
    return fail(g, TWS_ERR_INVALID, "terrain_rgba and mips must be 16-byte aligned");
  if (reinterpret_cast<uintptr_t>(flowmap) % 4 != 0)
    return fail(g, TWS_ERR_INVALID, "flowmap_rg16f must be 4-byte aligned");
  int w = g->W, h = g->H;
  for (int l = 1; l <= mip_levels; ++l) {
    if (w < 2 || h < 2) return fail(g, TWS_ERR_INVALID, "mip level smaller than 1x1");
    w /= 2;
    h /= 2;
  }
  TWS_CUDA(g, launch_export(g->b, g->d[g->cur], g->v, g->W, g->H, g->pitch, terrain_rgba, flowmap,
                            mip_levels, mips, g->stream),
           "export kernels");
  return TWS_OK;
}

TWS_API int tws_get_buffers(tws_grid* g, tws_buffers* out) {
  if (!g || !out) return TWS_ERR_INVALID;
  out->terrain = g->b;
  out->depth = g->d[g->cur];
  out->flux = g->f[g->cur];
  out->velocity = reinterpret_cast<const float*>(g->v);
  out->width = g->W;
  out->height = g->H;
  out->pitch = g->pitch;
  out->flux_storage = g->flux_storage;
  out->flux_scale = g->flux_scale;
  return TWS_OK;
}

TWS_API int tws_sync(tws_grid* g) {
  if (!g) return TWS_ERR_INVALID;
  if (const int rc = tws_io_wait(g)) return rc;
  TWS_CUDA(g, cudaMemcpyAsync(g->err_host, g->err, sizeof(int), cudaMemcpyDeviceToHost, g->stream),
           "error word copy");
  TWS_CUDA(g, cudaStreamSynchronize(g->stream), "sync");
  if (*g->err_host != kDevErrNone) {
    // report once; the word is cleared so the grid can be reloaded and reused
    *g->err_host = kDevErrNone;
    TWS_CUDA(g, cudaMemsetAsync(g->err, 0, sizeof(int), g->stream), "error word reset");
    return fail(g, TWS_ERR_TIMEOUT, "a kernel gave up waiting for its tile loads");
  }
  return TWS_OK;
}

}  // extern "C"

// ===========================================================================
// Batches: many grids advanced by one persistent launch per step.
//
// A chain is up to kChainSteps steps.  Before a chain the host writes the
// table of participating grids (their tensor maps, step arguments, buffers,
// ping-pong parity and the number of launches each takes) and the prefix of
// their tile counts into device memory with one stream-ordered copy, then
// replays a CUDA graph of the chain's launches.  The launches read everything
// from that table, so one graph per (variant, chain length) serves every
// composition of the batch: grids join and leave between chains (continuous
// batching) without re-capture.
// ===========================================================================

namespace {
constexpr int kChainSteps = 16;
}

struct tws_batch {
  int flux_storage = TWS_FLUX_F32;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<tws_grid*> grids;
  int variant = batch_variant_default();  // batched kernel variant
  bool use_graphs = true;
  int cap = 0;   // table capacity (grids)
  int ucap = 0;  // unit table capacity
  BatchGrid* d_grids = nullptr;
  BatchUnit* d_units = nullptr;
  // host staging, two slots so that filling one does not wait for the copy of the other
  BatchGrid* h_grids[2] = {nullptr, nullptr};
  BatchUnit* h_units[2] = {nullptr, nullptr};
  cudaEvent_t copied[2] = {nullptr, nullptr};
  int slot = 0;
  int uploaded_slot = -1;  // staging slot whose contents the device table holds
  int uploaded_m = 0;
  int uploaded_blocks = 0;
  struct Graph {
    int variant, launches, blocks;
    cudaGraphExec_t exec;
  };
  std::vector<Graph> graphs;
  uint64_t chains = 0, graph_launches = 0;
  int* d_err = nullptr;  // one device error word for every member while batched
  int uploaded_variant = -1;  // variant whose unit table the device holds
  int h_err = 0;
  std::string last_error;
};

namespace {

int bfail(tws_batch* b, int code, const std::string& msg) {
  if (b) b->last_error = msg;
  return code;
}

void drop_graphs(tws_batch* b) {
  for (auto& gr : b->graphs) cudaGraphExecDestroy(gr.exec);
  b->graphs.clear();
}

void free_units(tws_batch* b) {
  cudaFree(b->d_units);
  for (int s = 0; s < 2; ++s) {
    if (b->h_units[s]) cudaFreeHost(b->h_units[s]);
    b->h_units[s] = nullptr;
  }
  b->d_units = nullptr;
  b->ucap = 0;
  b->uploaded_slot = -1;  // the device table is gone
}

void free_table(tws_batch* b) {
  cudaFree(b->d_grids);
  for (int s = 0; s < 2; ++s) {
    if (b->h_grids[s]) cudaFreeHost(b->h_grids[s]);
    b->h_grids[s] = nullptr;
  }
  b->d_grids = nullptr;
  b->cap = 0;
  free_units(b);
}

// Grow the table to hold n grids (graphs reference the device arrays, so they
// are dropped when the arrays move).
int ensure_capacity(tws_batch* b, int n) {
  if (n <= b->cap) return TWS_OK;
  cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  free_table(b);
  int cap = 16;
  while (cap < n) cap *= 2;
  if (cudaMalloc(&b->d_grids, sizeof(BatchGrid) * cap) != cudaSuccess) {
    cudaGetLastError();
    free_table(b);
    return bfail(b, TWS_ERR_OOM, "batch table allocation failed");
  }
  for (int s = 0; s < 2; ++s) {
    if (cudaMallocHost(&b->h_grids[s], sizeof(BatchGrid) * cap) != cudaSuccess) {
      cudaGetLastError();
      free_table(b);
      return bfail(b, TWS_ERR_OOM, "batch staging allocation failed");
    }
  }
  b->cap = cap;
  return TWS_OK;
}

// Grow the unit table to at least n entries (a launch's CTA count), in powers
// of two so that a changing membership rarely reallocates it.
int ensure_units(tws_batch* b, int n) {
  if (n <= b->ucap) return TWS_OK;
  int cap = 256;
  while (cap < n) cap *= 2;
  n = cap;
  cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  free_units(b);
  if (cudaMalloc(&b->d_units, sizeof(BatchUnit) * n) != cudaSuccess) {
    cudaGetLastError();
    free_units(b);
    return bfail(b, TWS_ERR_OOM, "batch unit table allocation failed");
  }
  for (int s = 0; s < 2; ++s) {
    if (cudaMallocHost(&b->h_units[s], sizeof(BatchUnit) * n) != cudaSuccess) {
      cudaGetLastError();
      free_units(b);
      return bfail(b, TWS_ERR_OOM, "batch unit staging allocation failed");
    }
  }
  b->ucap = n;
  return TWS_OK;
}

int run_launches(tws_batch* b, int variant, int launches, int blocks) {
  for (int i = 0; i < launches; ++i) {
    cudaError_t e =
        launch_batch_step(variant, b->flux_storage, b->d_grids, b->d_units, i, blocks, b->stream);
    if (e != cudaSuccess) return bfail(b, TWS_ERR_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
  }
  return TWS_OK;
}

// CTAs per launch for a chain of `units` tiles: the next of 256, 288, ...,
// 480, 512, 576, ... (eight sizes per doubling), so that graphs stay reusable
// while the membership changes and at most an eighth of the CTAs launch only
// to return (a power of two wasted up to half: 2,496 of 8,192 on the 64-grid
// configuration).
int launch_blocks(int units) {
  int p = 256;
  while (2 * p <= units) p *= 2;  // p <= units < 2p (or units < 256)
  if (units <= p) return p;
  const int step = p / 8;
  return (units + step - 1) / step * step;
}

cudaGraphExec_t graph_for(tws_batch* b, int variant, int launches, int blocks) {
  for (auto& gr : b->graphs)
    if (gr.variant == variant && gr.launches == launches && gr.blocks == blocks) return gr.exec;
  if (prepare_batch_variant(variant, b->flux_storage) != cudaSuccess) return nullptr;
  cudaGraph_t graph = nullptr;
  if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return nullptr;
  const int rc = run_launches(b, variant, launches, blocks);
  const cudaError_t ee = cudaStreamEndCapture(b->stream, &graph);
  if (rc != TWS_OK || ee != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return nullptr;
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (b->graphs.size() >= 64) {  // bounded cache: drop the oldest graph
    cudaGraphExecDestroy(b->graphs.front().exec);
    b->graphs.erase(b->graphs.begin());
  }
  b->graphs.push_back({variant, launches, blocks, exec});
  return exec;
}

// One chain: grid i takes launches[i] launches of `variant` (K steps each).
int run_chain(tws_batch* b, int variant, const std::vector<int>& launches) {
  int k, tx, ty, sv;
  batch_variant_info(variant, &k, &tx, &ty, &sv);
  const int n = (int)b->grids.size();
  int rc = ensure_capacity(b, n);
  if (rc != TWS_OK) return rc;
  int units = 0, m = 0, max_l = 0;
  for (int i = 0; i < n; ++i) {
    if (launches[i] <= 0) continue;
    const tws_grid* g = b->grids[i];
    units += ((g->W + tx - 1) / tx) * ((g->H + ty - 1) / ty);
    max_l = std::max(max_l, launches[i]);
    ++m;
  }
  if (m == 0) return TWS_OK;
  const int blocks = launch_blocks(units);  // a power of two, so graphs stay reusable
  rc = ensure_units(b, blocks);
  if (rc != TWS_OK) return rc;
  // wait until the copy that last read this staging slot has completed
  const int s = b->slot;
  b->slot ^= 1;
  if (b->copied[s]) cudaEventSynchronize(b->copied[s]);
  BatchGrid* hg = b->h_grids[s];
  BatchUnit* hu = b->h_units[s];
  std::string why;
  m = 0;
  int u = 0;
  for (int i = 0; i < n; ++i) {
    if (launches[i] <= 0) continue;
    tws_grid* g = b->grids[i];
    BatchGrid& e = hg[m];
    std::memset(&e, 0, sizeof(e));  // padding too, so equal tables compare equal
    VariantMaps* maps = maps_for(g, sv, &why);
    if (!maps) return bfail(b, TWS_ERR_CUDA, why);
    if (!maps->on_device) {
      // written once per (grid, variant); the first chain's CTAs fence them
      CUtensorMap five[5] = {maps->b, maps->d[0], maps->d[1], maps->f[0], maps->f[1]};
      if (cudaMemcpyAsync(g->desc + 5 * sv, five, sizeof(five), cudaMemcpyHostToDevice,
                          b->stream) != cudaSuccess)
        return bfail(b, TWS_ERR_CUDA, "tensor map copy");
      maps->on_device = true;
      maps->fresh = true;
    }
    e.tm = g->desc + 5 * sv;
    e.fence = maps->fresh ? 1 : 0;
    maps->fresh = false;
    e.a = make_step_args(g);
    e.a.err = b->d_err;
    e.d[0] = g->d[0];
    e.d[1] = g->d[1];
    e.f[0] = g->f[0];
    e.f[1] = g->f[1];
    e.v = g->v;
    e.cur = g->cur;
    e.launches = launches[i];
    ++m;
  }
  // The units: every member's interior tiles first, then the tiles at the
  // members' edges, so that the CTAs resident on an SM at a time mostly run
  // one of the two code paths (the edge path is separate code, and mixing
  // the two stalled the schedulers on instruction fetch).  Interior is the
  // kernel's test: the tile's b/d box (halo 2K rounded up to 4 in x, 2K in y)
  // lies inside the grid.
  const int hx = (2 * k + 3) / 4 * 4, hy = 2 * k;
  for (int pass = 0; pass < 2; ++pass) {
    m = 0;
    for (int i = 0; i < n; ++i) {
      if (launches[i] <= 0) continue;
      const tws_grid* g = b->grids[i];
      const int meta = launches[i] | (g->cur << 30);
      for (int y0 = 0; y0 < g->H; y0 += ty)
        for (int x0 = 0; x0 < g->W; x0 += tx) {
          const bool interior = x0 - hx >= 0 && y0 - hy >= 0 && x0 + tx + hx <= g->W &&
                                y0 + ty + hy <= g->H;
          if (interior == (pass == 0)) hu[u++] = BatchUnit{m, x0, y0, meta};
        }
      ++m;
    }
  }
  for (; u < blocks; ++u) hu[u] = BatchUnit{0, 0, 0, 0};  // CTAs past the units return
  // Upload the table unless it equals the one the device already holds (the
  // same members, launch counts and parity: consecutive chains of a steady
  // batch with an even number of launches).  The units follow from the
  // members and the launch size.
  const int prev = b->uploaded_slot;
  const bool same = prev >= 0 && b->uploaded_m == m && b->uploaded_blocks == blocks &&
                    b->uploaded_variant == variant &&
                    std::memcmp(hg, b->h_grids[prev], sizeof(BatchGrid) * m) == 0;
  if (same) {
    b->slot = prev ^ 1;  // keep the uploaded copy in its slot for the next comparison
  } else {
    b->uploaded_slot = -1;  // until the copies below are queued
    if (cudaMemcpyAsync(b->d_grids, hg, sizeof(BatchGrid) * m, cudaMemcpyHostToDevice,
                        b->stream) != cudaSuccess ||
        cudaMemcpyAsync(b->d_units, hu, sizeof(BatchUnit) * blocks, cudaMemcpyHostToDevice,
                        b->stream) != cudaSuccess ||
        (!b->copied[s] &&
         cudaEventCreateWithFlags(&b->copied[s], cudaEventDisableTiming) != cudaSuccess) ||
        cudaEventRecord(b->copied[s], b->stream) != cudaSuccess)
      return bfail(b, TWS_ERR_CUDA, "batch table upload");
    b->uploaded_slot = s;
    b->uploaded_m = m;
    b->uploaded_blocks = blocks;
    b->uploaded_variant = variant;
  }
  cudaGraphExec_t exec = b->use_graphs ? graph_for(b, variant, max_l, blocks) : nullptr;
  if (exec) {
    if (cudaGraphLaunch(exec, b->stream) != cudaSuccess)
      return bfail(b, TWS_ERR_CUDA, "graph launch failed");
    count_launch((uint64_t)max_l);
    ++b->graph_launches;
  } else {
    rc = run_launches(b, variant, max_l, blocks);
    if (rc != TWS_OK) return rc;
  }
  ++b->chains;
  // each launch flips a grid's ping-pong buffer once
  for (int i = 0; i < n; ++i)
    if (launches[i] > 0) b->grids[i]->cur ^= (launches[i] & 1);
  return TWS_OK;
}

// Advance member i by steps[i] steps (chains of up to kChainSteps).
int batch_advance(tws_batch* b, std::vector<int> left) {
  int k;
  batch_variant_info(b->variant, &k, nullptr, nullptr, nullptr);
  const int n = (int)b->grids.size();
  const int per_chain = std::max(1, kChainSteps / k);  // launches per chain
  std::vector<int> launches(n);
  for (;;) {
    bool work = false;
    for (int i = 0; i < n; ++i) {
      launches[i] = std::min(left[i] / k, per_chain);
      work |= launches[i] > 0;
    }
    if (!work) break;
    const int rc = run_chain(b, b->variant, launches);
    if (rc != TWS_OK) return rc;
    for (int i = 0; i < n; ++i) left[i] -= launches[i] * k;
  }
  // steps left over when K does not divide a grid's count: one-step launches
  bool any = false;
  for (int i = 0; i < n; ++i) any |= left[i] > 0;
  if (any) {
    int k1 = -1;
    for (int v = 0; v < batch_variant_count(); ++v) {
      int kv;
      batch_variant_info(v, &kv, nullptr, nullptr, nullptr);
      if (kv == 1) {
        k1 = v;
        break;
      }
    }
    if (k1 < 0) return bfail(b, TWS_ERR_UNSUPPORTED, "no one-step batched variant");
    return run_chain(b, k1, left);
  }
  return TWS_OK;
}

}  // namespace

extern "C" {

TWS_API int tws_batch_create(int flux_storage, void* stream, tws_batch** out) {
  if (!out || (flux_storage != TWS_FLUX_F32 && flux_storage != TWS_FLUX_F16)) return TWS_ERR_INVALID;
  *out = nullptr;
  tws_batch* b = new (std::nothrow) tws_batch();
  if (!b) return TWS_ERR_OOM;
  b->flux_storage = flux_storage;
  if (stream) {
    b->stream = static_cast<cudaStream_t>(stream);
  } else {
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete b;
      return TWS_ERR_CUDA;
    }
    b->own_stream = true;
  }
  if (cudaMalloc(&b->d_err, sizeof(int)) != cudaSuccess ||
      cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream) != cudaSuccess) {
    cudaGetLastError();
    if (b->own_stream) cudaStreamDestroy(b->stream);
    cudaFree(b->d_err);
    delete b;
    return TWS_ERR_CUDA;
  }
  *out = b;
  return TWS_OK;
}

TWS_API int tws_batch_remove(tws_batch* b, tws_grid* g) {
  if (!b || !g || g->batch != b) return bfail(b, TWS_ERR_INVALID, "grid is not in this batch");
  cudaStreamSynchronize(b->stream);
  b->grids.erase(std::find(b->grids.begin(), b->grids.end(), g));
  g->stream = g->home_stream;
  g->batch = nullptr;
  return TWS_OK;
}

TWS_API int tws_batch_destroy(tws_batch* b) {
  if (!b) return TWS_ERR_INVALID;
  while (!b->grids.empty()) tws_batch_remove(b, b->grids.back());
  cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  free_table(b);
  for (int s = 0; s < 2; ++s)
    if (b->copied[s]) cudaEventDestroy(b->copied[s]);
  cudaFree(b->d_err);
  if (b->own_stream) cudaStreamDestroy(b->stream);
  delete b;
  return TWS_OK;
}

TWS_API int tws_batch_add(tws_batch* b, tws_grid* g) {
  if (!b || !g) return TWS_ERR_INVALID;
  if (g->batch) return bfail(b, TWS_ERR_INVALID, "grid already belongs to a batch");
  if (g->flux_storage != b->flux_storage)
    return bfail(b, TWS_ERR_INVALID, "grid flux storage differs from the batch's");
  // the grid's queued work finishes first; from now on it is ordered on the batch stream
  if (cudaStreamSynchronize(g->stream) != cudaSuccess)
    return bfail(b, TWS_ERR_CUDA, "grid stream failed");
  g->home_stream = g->stream;
  g->stream = b->stream;
  g->batch = b;
  b->grids.push_back(g);
  return TWS_OK;
}

TWS_API int tws_batch_size(tws_batch* b) { return b ? (int)b->grids.size() : 0; }

TWS_API int tws_batch_variant_count(void) { return batch_variant_count(); }

TWS_API int tws_batch_variant_info(int i, int* k, int* tx, int* ty) {
  if (i < 0 || i >= batch_variant_count()) return TWS_ERR_INVALID;
  batch_variant_info(i, k, tx, ty, nullptr);
  return TWS_OK;
}

TWS_API int tws_batch_set_variant(tws_batch* b, int variant) {
  if (!b || variant < 0 || variant >= batch_variant_count())
    return bfail(b, TWS_ERR_INVALID, "no such batched variant");
  b->variant = variant;
  return TWS_OK;
}

TWS_API int tws_batch_use_graphs(tws_batch* b, int enable) {
  if (!b) return TWS_ERR_INVALID;
  b->use_graphs = enable != 0;
  return TWS_OK;
}

TWS_API int tws_batch_step(tws_batch* b, int nsteps) {
  if (!b || nsteps < 0) return bfail(b, TWS_ERR_INVALID, "bad step count");
  return batch_advance(b, std::vector<int>(b->grids.size(), nsteps));
}

TWS_API int tws_batch_step_each(tws_batch* b, const int* nsteps, int n) {
  if (!b || !nsteps || n != (int)b->grids.size()) return bfail(b, TWS_ERR_INVALID, "bad step list");
  for (int i = 0; i < n; ++i)
    if (nsteps[i] < 0) return bfail(b, TWS_ERR_INVALID, "negative step count");
  return batch_advance(b, std::vector<int>(nsteps, nsteps + n));
}

TWS_API int tws_batch_autotune(tws_batch* b, int trial_steps, int* chosen) {
  if (!b || trial_steps < 1) return bfail(b, TWS_ERR_INVALID, "trial_steps must be positive");
  const int n = (int)b->grids.size();
  if (n == 0) return bfail(b, TWS_ERR_INVALID, "empty batch");
  cudaStreamSynchronize(b->stream);
  // save every member's state; the trials run on it and it is restored after
  struct Saved {
    float* d;
    void* f;
    float2* v;
    int cur;
  };
  std::vector<Saved> saved(n);
  for (int i = 0; i < n; ++i) {
    tws_grid* g = b->grids[i];
    const size_t cells = (size_t)g->pitch * g->H, fb = flux_bytes_per_cell(g->flux_storage);
    saved[i].cur = g->cur;
    if (cudaMallocAsync(&saved[i].d, cells * 4, b->stream) != cudaSuccess ||
        cudaMallocAsync(&saved[i].f, cells * fb, b->stream) != cudaSuccess ||
        cudaMallocAsync(&saved[i].v, cells * 8, b->stream) != cudaSuccess)
      return bfail(b, TWS_ERR_OOM, "autotune state copy");
    cudaMemcpyAsync(saved[i].d, g->d[g->cur], cells * 4, cudaMemcpyDeviceToDevice, b->stream);
    cudaMemcpyAsync(saved[i].f, g->f[g->cur], cells * fb, cudaMemcpyDeviceToDevice, b->stream);
    cudaMemcpyAsync(saved[i].v, g->v, cells * 8, cudaMemcpyDeviceToDevice, b->stream);
  }
  auto restore = [&]() {
    for (int i = 0; i < n; ++i) {
      tws_grid* g = b->grids[i];
      const size_t cells = (size_t)g->pitch * g->H, fb = flux_bytes_per_cell(g->flux_storage);
      g->cur = saved[i].cur;
      cudaMemcpyAsync(g->d[g->cur], saved[i].d, cells * 4, cudaMemcpyDeviceToDevice, b->stream);
      cudaMemcpyAsync(g->f[g->cur], saved[i].f, cells * fb, cudaMemcpyDeviceToDevice, b->stream);
      cudaMemcpyAsync(g->v, saved[i].v, cells * 8, cudaMemcpyDeviceToDevice, b->stream);
    }
  };
  const int steps = (trial_steps + 2 * kChainSteps - 1) / (2 * kChainSteps) * (2 * kChainSteps);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int saved_variant = b->variant;
  float best_ms = 1e30f;
  int best = saved_variant, rc = TWS_OK;
  for (int v = 0; v < batch_variant_count() && rc == TWS_OK; ++v) {
    float vbest = 1e30f;
    for (int rep = 0; rep < 2 && rc == TWS_OK; ++rep) {
      restore();
      b->variant = v;
      cudaEventRecord(e0, b->stream);
      rc = batch_advance(b, std::vector<int>(n, steps));
      cudaEventRecord(e1, b->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = TWS_ERR_CUDA;
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      vbest = std::min(vbest, ms);
    }
    if (vbest < best_ms) {
      best_ms = vbest;
      best = v;
    }
  }
  restore();
  for (int i = 0; i < n; ++i) {
    cudaFreeAsync(saved[i].d, b->stream);
    cudaFreeAsync(saved[i].f, b->stream);
    cudaFreeAsync(saved[i].v, b->stream);
  }
  cudaStreamSynchronize(b->stream);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->variant = rc == TWS_OK ? best : saved_variant;
  if (chosen) *chosen = b->variant;
  return rc;
}

TWS_API int tws_batch_sync(tws_batch* b) {
  if (!b) return TWS_ERR_INVALID;
  if (cudaMemcpyAsync(&b->h_err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    return bfail(b, TWS_ERR_CUDA, "batch sync");
  if (b->h_err != kDevErrNone) {
    b->h_err = kDevErrNone;
    if (cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream) != cudaSuccess)
      return bfail(b, TWS_ERR_CUDA, "error word reset");
    return bfail(b, TWS_ERR_TIMEOUT, "a batched kernel gave up waiting for its tile loads");
  }
  return TWS_OK;
}

TWS_API void* tws_batch_stream(tws_batch* b) { return b ? (void*)b->stream : nullptr; }

TWS_API const char* tws_batch_last_error(tws_batch* b) {
  return b ? b->last_error.c_str() : "null batch";
}

TWS_API double tws_grid_bytes(int width, int height, int flux_storage) {
  if (width < 1 || height < 1) return 0.0;
  const double cells = (double)((width + 31) / 32 * 32) * height;
  return cells * (4.0 + 8.0 + 2.0 * flux_bytes_per_cell(flux_storage) + 8.0) +
         sizeof(double) * (volume_partials_needed() + 1) + sizeof(int);
}

TWS_API int tws_batch_stats(tws_batch* b, uint64_t* chains, uint64_t* graph_launches) {
  if (!b) return TWS_ERR_INVALID;
  if (chains) *chains = b->chains;
  if (graph_launches) *graph_launches = b->graph_launches;
  return TWS_OK;
}

}  // extern "C"
