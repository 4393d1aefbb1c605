// tws_internal.h -- shared declarations of the libtws implementation.
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/tws.h"
#include "../../include/tws_testing.h"

namespace tws {

// ---------------------------------------------------------------------------
// Per-step source in the form the kernels read (bounding box precomputed).
struct DevSource {
  int kind;
  float cx, cy, radius, rate;
  int icx, icy, ir;    // DISK: integer centre and radius
  int bx0, by0, bx1, by1;  // inclusive bounding box of the cells it can touch
};

// Everything a step launch needs besides the tensor maps.
struct StepArgs {
  int W, H, pitch;
  float kf, ka, c;
  int closed;
  int nsrc;
  DevSource src[TWS_MAX_SOURCES];
  float* d_out;
  void* f_out;
  float2* v_out;
  float flux_scale;      // F16 storage: stored = f * flux_scale
  float flux_inv_scale;  // F16 storage: f = stored * flux_inv_scale
  int* err;              // device error word (bounded-wait time-outs)
  long long wait_cycles; // bounded waits give up after this many SM clocks
  int drop_loads;        // test hook: tile loads arm their barrier but issue no copy
  int* queue;            // the sweep kernel's work queue: next unit, warps done (zero
                         // between launches; the last warp of a launch resets it)
};

// Kernel variants (temporal block depth K x tile).
struct StepVariant {
  int k;      // steps per launch
  int tx, ty; // interior tile
  int stages; // 1: one CTA per tile; 2: persistent CTAs, next tile prefetched
  int kind;   // kKindTile (TMA-staged tiles), kKindStream (register streaming, K = 1)
              // or kKindSweep (row sweep over column strips, K time levels in registers)
  int ry;     // kKindStream, kKindSweep: rows per warp strip
  int hx;     // x halo of the b/d boxes (2K rounded up to 4 floats)
  int bw, bh; // b/d box
  int fw, fh; // flux box
  int sw;     // F16 staging width in cells (whole pairs)
  int uni;    // unified layout: the flux box is the b/d box
  int ring;   // kKindSweep: rows in each lane's load ring
  int ry_tail; // kKindSweep: rows of the short bands that end the work queue (0: none)
  size_t smem;
};

enum : int { kKindTile = 0, kKindStream = 1, kKindSweep = 2 };

// One member grid of a batch as the batched kernel reads it from device
// memory: its tensor maps, its step arguments and its buffers.  The maps are
// not in this table (which the host rewrites between chains) but in a block
// of the grid's own memory written once per kernel variant: tm[0] terrain,
// tm[1 + i] depth buffer i, tm[3 + i] flux buffer i.  A CTA makes the
// tensor-map proxy re-read them (an acquire fence, which costs a descriptor
// fetch per tile) only in the first chain after they were written: `fence`.
struct alignas(16) BatchGrid {
  const CUtensorMap* tm;
  int fence;
  int pad0_;
  StepArgs a;     // W, H, pitch, constants, sources, flux scale, error word
  float* d[2];
  void* f[2];
  float2* v;
  // The kernel takes both from the unit records; here they make a changed
  // chain compare unequal with the table the device holds.
  int cur;        // buffer holding the state when the chain starts
  int launches;   // launches of this chain that advance this grid
};

// One work unit (tile) of a batched launch, as the batched kernel reads it:
// its grid (index into the BatchGrid table), tile origin, and meta =
// launches this chain gives the grid | (the grid's buffer parity at the chain
// start) << 30.  Entries past the chain's units have meta = 0.
struct BatchUnit {
  int grid, x0, y0, meta;
};

// Batched kernel variants (K steps per launch, tile) and their launcher.
// Launch `launch_idx` of a chain runs CTA u on units[u] (`blocks` CTAs, at
// least the chain's units) and advances a grid iff launch_idx < its launches.
int batch_variant_count();
int batch_variant_default();  // two steps per launch, unified 32x32 tiles
void batch_variant_info(int i, int* k, int* tx, int* ty, int* step_variant);
cudaError_t prepare_batch_variant(int variant, int flux_storage);  // outside any capture
cudaError_t launch_batch_step(int variant, int flux_storage, const BatchGrid* grids,
                              const BatchUnit* units, int launch_idx, int blocks, cudaStream_t s);

// Device error codes written to StepArgs::err.
enum : int { kDevErrNone = 0, kDevErrWaitTimeout = 1 };

// Default limit of a bounded tile-load wait: about two seconds at 2 GHz, far
// beyond any real load, short enough that a lost load ends the kernel.
constexpr long long kDefaultWaitCycles = 4000000000LL;

// Host helpers implemented in tws_step.cu.
int step_variant_count();
const StepVariant& step_variant(int i);
int step_variant_for(int k, int flux_storage);
// The automatic choice for grids of at least kLargeGridCells cells (FP16
// flux: kLargeF16Cells), or -1.
constexpr long long kLargeGridCells = 12LL << 20;
constexpr long long kLargeF16Cells = 32LL << 20;
int step_variant_large_grid(int flux_storage, int W, int H);
// Tile variants read through the tensor maps, stream variants through the
// raw pointers (b, d, f of the current state).
cudaError_t launch_step(int variant, int flux_storage, const CUtensorMap* tm_b,
                        const CUtensorMap* tm_d, const CUtensorMap* tm_f, const float* b,
                        const float* d, const void* f, const StepArgs& a, cudaStream_t s);
// tws_sweep.cu: K = 2..4 steps per launch, `rows` rows per warp band (the
// last bands `tail_rows` rows when it is above 0), a ring of `ring` rows per
// lane (4)
cudaError_t launch_sweep_step(int k, int rows, int tail_rows, int ring, int flux_storage,
                              const float* b,
                              const float* d, const void* f, const StepArgs& a, cudaStream_t s);
constexpr int kSweepCtaThreads = 128;  // four warps, each its own sweep
size_t sweep_smem_bytes(int k, int flux_storage, int ring);
int sweep_valid_columns(int k);
// tws_stream.cu
cudaError_t launch_stream_step(int ry, int flux_storage, const float* b, const float* d,
                               const void* f, const StepArgs& a, cudaStream_t s);
cudaError_t encode_step_maps(int variant, int flux_storage, int W, int H, int pitch,
                             const float* b, const float* d, const void* f, CUtensorMap* tm_b,
                             CUtensorMap* tm_d, CUtensorMap* tm_f, std::string* why);

// tws_resident.cu: the whole grid in the shared memory of one cluster of up
// to kResidentMaxCluster CTAs, up to kResidentMaxSteps steps per launch.
constexpr int kResidentMaxCluster = 16;
constexpr int kResidentMaxSteps = 4096;
// cudaSuccess if a W x H grid fits a cluster of `ctas` CTAs (0: the automatic
// size, returned in *chosen) and the device can run that cluster
cudaError_t resident_supported(int W, int H, int flux_storage, int ctas, int* chosen);
cudaError_t launch_resident(int flux_storage, int ctas, const float* b, const float* d,
                            const void* f, const StepArgs& a, int nsteps, cudaStream_t s);

// tws_aux.cu
cudaError_t launch_apply_source(float* d, int W, int H, int pitch, const DevSource& s,
                                cudaStream_t st);
cudaError_t launch_volume(const float* d, int W, int H, int pitch, double cell_area,
                          double* partials, int max_partials, double* out, cudaStream_t st);
int volume_partials_needed();
cudaError_t launch_generate_scene(uint64_t seed, int W, int H, int pitch, float height_scale,
                                  float fill, float* b, float* d, cudaStream_t st);
cudaError_t launch_reference_scene(uint32_t seed, int generation, int W, int H, int pitch,
                                   float height_scale, float* b, float* d, cudaStream_t st);
cudaError_t launch_flux_to_f32(const void* f, int flux_storage, float inv_scale, int W, int H,
                               int pitch, float* out_packed, cudaStream_t st);
cudaError_t launch_flux_from_f32(const float* in_packed, int flux_storage, float scale, int W,
                                 int H, int pitch, void* f, cudaStream_t st);
// Up to four row copies between packed arrays and the pitched state in one
// launch on the SMs (device-to-device copies on the copy engines are several
// times slower); a null source writes zeros.  Pitches and row lengths in
// floats; `vec` is filled by the launcher.
struct StageRows {
  const float* src[4];
  float* dst[4];
  int row_floats[4], src_pitch[4], dst_pitch[4], vec[4];
  int n;
  void add(const float* s, int sp, float* d, int dp, int floats) {
    src[n] = s;
    dst[n] = d;
    src_pitch[n] = sp;
    dst_pitch[n] = dp;
    row_floats[n] = floats;
    vec[n] = 1;
    ++n;
  }
};
cudaError_t launch_stage_rows(const StageRows& sr, int H, cudaStream_t st);

// tws_export.cu
cudaError_t launch_surface(const float* b, const float* d, const float2* v, int W, int H,
                           int pitch, const tws_surface_out& o, cudaStream_t s);
cudaError_t launch_export(const float* b, const float* d, const float2* v, int W, int H,
                          int pitch, float* terrain_rgba, uint16_t* flowmap, int mip_levels,
                          float* mips, cudaStream_t s);

DevSource make_dev_source(const tws_source& s);
void count_launch(uint64_t n = 1);

}  // namespace tws
