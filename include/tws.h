/* tws.h -- C ABI of the GB300 virtual-pipe shallow-water step.
 *
 * This is the drop-in boundary for the simulation half of terrainwatersim's
 * `Terrain` class (terrainwatersim/source/scene/Terrain.h:15-153).  The
 * reference keeps its state in three OpenGL textures and advances it with two
 * compute-shader dispatches per step; this library keeps the same state in
 * device buffers on one GPU and advances it with hand-written sm_103a kernels.
 *
 * Conventions
 *   - Every call returns an int status: TWS_OK (0) or a negative TWS_ERR_*.
 *     tws_error_string() names a code; tws_last_error() gives the message of
 *     the last failure on a grid.  No C++ exception crosses this boundary.
 *   - Host arrays are row-major, tightly packed, `width` floats per row.
 *     Flux is 4 floats per cell in the reference's channel order
 *     (+x, -x, +y, -y) = (.x, .y, .z, .w) of the Flow texture
 *     (flowUpdate.comp:44-47); velocity ("flow map") is 2 floats per cell
 *     (flowApply.comp:45-46).
 *   - Calls on one grid are enqueued on that grid's CUDA stream and are
 *     asynchronous unless stated.  One grid must not be used from two host
 *     threads at once; distinct grids are independent.
 *   - There is no CPU fallback: without a usable sm_103a device, tws_create
 *     fails with TWS_ERR_CUDA.
 */
#ifndef TWS_H_
#define TWS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TWS_API __attribute__((visibility("default")))

/* ---- status codes ---------------------------------------------------- */
#define TWS_OK 0
#define TWS_ERR_INVALID -1     /* bad argument (size, pointer, enum)        */
#define TWS_ERR_CUDA -2        /* a CUDA runtime/driver call failed         */
#define TWS_ERR_OOM -3         /* device allocation failed                  */
#define TWS_ERR_TIMEOUT -4     /* a device-side bounded wait gave up        */
#define TWS_ERR_UNSUPPORTED -5 /* option not built into this library        */
#define TWS_ERR_BUSY -6        /* admission refused (serving loop)          */
#define TWS_ERR_TOO_LARGE -7   /* input exceeds a fixed-size scratch array  */

/* ---- enums ------------------------------------------------------------ */
#define TWS_BOUNDARY_CLOSED 0 /* zero flux across the grid border          */
#define TWS_BOUNDARY_OPEN 1   /* reference semantics: off-grid cells read  */
                              /* as zero, water drains off the edge        */
                              /* (GL imageLoad out of range, flowUpdate.comp:18,29-32) */
#define TWS_FLUX_F32 0        /* flux stored as 4 x float per cell          */
#define TWS_FLUX_F16 1        /* flux stored as 4 x half per cell, times a  */
                              /* per-grid power-of-two scale               */
#define TWS_SOURCE_DISK 0     /* uniform disk: +rate metres per step inside */
#define TWS_SOURCE_BRUSH 1    /* reference radial brush, waterBrush.comp:26-28 */

#define TWS_MAX_SOURCES 8

/* ---- parameters --------------------------------------------------------
 * The three per-step constants of the reference's SimulationParameters
 * uniform block (terrainwatersim/shader/simulationCommon.glsl:1-13).       */
typedef struct tws_sim_params {
  float flow_friction_per_step;      /* Kf, FlowFriction_perStep            */
  float water_acceleration_per_step; /* Ka, WaterAcceleration_perStep       */
  float cell_area_inv_time_scaled;   /* C,  CellAreaInv_timeScaled          */
  float cell_area;                   /* l*l, scales tws_volume               */
  int boundary;                      /* TWS_BOUNDARY_*                       */
} tws_sim_params;

/* Physical form: Kf = damping_per_step, Ka = dt*g*A/l, C = dt/l^2 (the
 * formulas stated in simulationCommon.glsl:5-11), evaluated in double and
 * rounded to float once. */
TWS_API int tws_params_physical(double dt, double gravity, double pipe_area, double cell_size,
                                double damping_per_step, int boundary, tws_sim_params* out);

/* Reference form: the derivations of Terrain::SetSimulationStepsPerSecond,
 * SetFlowDamping and SetFlowAcceleration (Terrain.cpp:175-198):
 * Kf = pow(damping, step), Ka = step*acceleration*cellDistance,
 * C = step/cellDistance^2, with step = 1/steps_per_second and
 * cellDistance = grid_world_size/grid_resolution. */
TWS_API int tws_params_reference(float steps_per_second, float flow_damping,
                                 float flow_acceleration, float grid_world_size,
                                 unsigned grid_resolution, int boundary, tws_sim_params* out);

/* A water source.  DISK (the benchmark's rain): every cell whose integer
 * offset (x-cx, y-cy) satisfies dx*dx+dy*dy <= radius*radius gains `rate`
 * metres (cx, cy, radius are whole cells).  The FP32 sum d + rate is rounded
 * without bias: down or up to a neighbouring float with the probability that
 * makes its expectation exact, decided by a hash of the cell and the bits of
 * d (deterministic), so long rainy runs conserve volume.  BRUSH (the reference's brush,
 * waterBrush.comp:26-28): d += saturate(1 - |(cx,cy)-(x,y)|^2 / radius) * rate,
 * where radius holds BrushSizeSq and rate BrushIntensity. */
typedef struct tws_source {
  int kind;
  float cx, cy;
  float radius;
  float rate;
} tws_source;

typedef struct tws_grid tws_grid; /* opaque */

/* Device view of a grid's state, valid until the next tws_step or
 * tws_destroy (the step ping-pongs depth and flux).  Rows are `pitch`
 * elements apart. */
typedef struct tws_buffers {
  const float* terrain;  /* b, float per cell                                */
  const float* depth;    /* d, float per cell                                */
  const void* flux;      /* 4 x float (F32) or 4 x half (F16) per cell       */
  const float* velocity; /* 2 x float per cell (flow map, last step)         */
  int width, height, pitch;
  int flux_storage;      /* TWS_FLUX_*                                       */
  float flux_scale;      /* F16: stored = flux * flux_scale (power of two)  */
} tws_buffers;

/* ---- lifecycle -----------------------------------------------------------
 * Replaces Terrain::Terrain + CreateHeightmapFromNoiseAndResetSim's texture
 * allocation (Terrain.cpp:21-132, 200-238).  `stream` is a cudaStream_t
 * (NULL: the library creates one).  State starts as b = d = f = v = 0.
 * 1 <= width <= 2^20, 1 <= height <= 2^19. */
TWS_API int tws_create(int width, int height, const tws_sim_params* params, int flux_storage,
                       void* stream, tws_grid** out);
/* Replaces Terrain::~Terrain (Terrain.cpp:134-148).  Waits for the grid's
 * asynchronous host copies (tws_upload_async / tws_download_async), which may
 * still read or write caller arrays; device memory returns to the pool in
 * stream order, without waiting for queued steps. */
TWS_API int tws_destroy(tws_grid* grid);

/* Reset from host arrays: terrain (required), depth (NULL -> 0), flux
 * (NULL -> 0); velocity is cleared.  Replaces the uploads of
 * CreateHeightmapFromNoiseAndResetSim (Terrain.cpp:223, 230-234).
 * Synchronous with respect to the host arrays (they may be reused on return). */
TWS_API int tws_upload(tws_grid* grid, const float* terrain, const float* depth,
                       const float* flux);
/* Same, from tightly packed device arrays. */
TWS_API int tws_upload_device(tws_grid* grid, const float* terrain, const float* depth,
                              const float* flux);

/* Reset to the synthetic benchmark scene, generated on the device: seeded
 * PCG32 value-noise fBm terrain scaled to [0, height_scale), depth
 * max(0, fill - b), flux and velocity zero.  Stands in for
 * CreateHeightmapFromNoiseAndResetSim (Terrain.cpp:200-238), whose own noise
 * generator is not the benchmark's. */
TWS_API int tws_generate_scene(tws_grid* grid, uint64_t seed, float height_scale, float fill);

/* Reset to the reference's own scene, Terrain::CreateHeightmapFromNoiseAndResetSim
 * (Terrain.cpp:200-238), generated on the device: terrain from the reference's
 * value noise (NoiseGenerator.cpp:12-97; octaves 2..10, persistence 0.43,
 * periodic) scaled to height_scale (the reference's default: 300), depth
 * max(0, (0.45 - r^4 * 800) * height_scale - b) with r the distance from the
 * grid centre in grid units, flux and velocity zero.  The noise table is the
 * one the reference's Random.cpp gives after Init(seed) (the application uses
 * TWS_REFERENCE_NOISE_SEED, Application.cpp:57) and `generation` earlier
 * scenes (0: the first, each reset draws a new table).  The reference's grid
 * is square; a W x H grid uses 1/(W-1) and 1/(H-1) per axis.  W, H >= 2. */
#define TWS_REFERENCE_NOISE_SEED 231656522u
TWS_API int tws_generate_reference_scene(tws_grid* grid, uint32_t seed, int generation,
                                         float height_scale);

/* Rain disks of the synthetic benchmark scene: `count` DISK sources of the
 * given radius and rate, centres drawn from the PCG32 stream
 * (seed, 1000 + k): cx = r + u0 % (W - 2r), cy = r + u1 % (H - 2r) (grid
 * centre if the disk does not fit).  Host-only; no counterpart in the
 * reference, whose water source is the interactive brush. */
TWS_API int tws_scene_rain_disks(uint64_t seed, int width, int height, int radius, float rate,
                                 int count, tws_source* out);

/* Replaces the SimulationParameters setters (Terrain.cpp:175-198). */
TWS_API int tws_set_params(tws_grid* grid, const tws_sim_params* params);

/* Per-step sources, applied at the start of every step inside the step
 * kernel (n <= TWS_MAX_SOURCES; n = 0 clears). */
TWS_API int tws_set_sources(tws_grid* grid, const tws_source* sources, int n);

/* One-shot source applied now, before the next step: replaces
 * Terrain::ApplyRadialWaterBrush's dispatch (Terrain.cpp:150-168). */
TWS_API int tws_apply_source(tws_grid* grid, const tws_source* source);

/* Steps per launch of the fused kernel (temporal blocking depth): 1 (plain),
 * 2, 3 or 4.  0 selects the library's choice for this grid size.  Results do
 * not depend on it (bit-identical). */
TWS_API int tws_set_steps_per_launch(tws_grid* grid, int steps_per_launch);

/* Kernel variants: each is a temporal depth K (steps per launch), an output
 * tile and a pipeline depth (1: one CTA per tile; 2: persistent CTAs that
 * prefetch their next tile while computing).  tws_variant_info describes
 * variant i (any pointer may be NULL); returns TWS_ERR_INVALID past the last
 * one. */
TWS_API int tws_variant_count(void);
TWS_API int tws_variant_info(int variant, int* steps_per_launch, int* tile_x, int* tile_y,
                             int* stages, size_t* shared_bytes);
/* The kind of kernel variant i, or TWS_ERR_INVALID past the last one:
 * TWS_VARIANT_TILE (TMA-staged tiles: tile_x x tile_y output cells per CTA),
 * TWS_VARIANT_STREAM (register streaming, one step: tile_x columns per warp
 * walking tile_y rows) or TWS_VARIANT_SWEEP (a warp sweeps a strip of tile_x
 * output columns down a band of tile_y rows, the steps' time levels in
 * registers).  Only the tile variants wait on barriers that
 * tws_set_wait_limit bounds. */
#define TWS_VARIANT_TILE 0
#define TWS_VARIANT_STREAM 1
#define TWS_VARIANT_SWEEP 2
TWS_API int tws_variant_kind(int variant);
/* Rows of the short bands that end a sweep variant's work queue (its other
 * bands are tile_y rows; the short ones are the grid's last rows, about one
 * unit per resident warp), 0 for none and for other kinds, or
 * TWS_ERR_INVALID past the last variant. */
TWS_API int tws_variant_tail_rows(int variant);

/* Pin a variant for this grid (-1: automatic -- the tuned choice for this
 * grid shape if tws_autotune ran for one, else the steps-per-launch setting). */
TWS_API int tws_set_variant(tws_grid* grid, int variant);
/* The variant that tws_step launches for this grid now: the pinned one, the
 * tuned one, or the automatic choice for its size and flux storage (a call's
 * remainder of fewer steps than the variant's depth runs a shallower tile
 * variant).  The resident kernel (tws_set_resident) is not a variant. */
TWS_API int tws_current_variant(tws_grid* grid, int* variant);

/* Failure detection (no reference counterpart: the reference's shaders have
 * no waits that can run out).  A step kernel waits on a barrier for each of
 * its tile loads; the wait gives up after `sm_cycles` SM clocks (0: the
 * default, about two seconds), sets the grid's error word and returns
 * without writing that tile.  The next tws_sync then reports TWS_ERR_TIMEOUT
 * once and clears the word; the state is undefined after it and must be
 * uploaded again, and the context stays usable.  (The test hook that makes
 * the waits run out is declared in tws_testing.h, not here.) */
TWS_API int tws_set_wait_limit(tws_grid* grid, long long sm_cycles);

/* Autotuner: times every variant for `trial_steps` steps on this grid's
 * current state (restored afterwards, so the simulation is unchanged), picks
 * the fastest per cell-step, pins it on this grid and records it for every
 * later grid of the same width, height and flux storage in this process.
 * Where the grid fits the resident kernel (below), that is timed too; if it
 * is fastest, it runs every later tws_step call of at least 16 steps on
 * grids of this shape, and the fastest tiled variant the shorter calls.
 * Synchronous.  `chosen` (may be NULL) receives the variant index, or
 * TWS_VARIANT_RESIDENT if the resident kernel was fastest.  No counterpart
 * in the reference. */
#define TWS_VARIANT_RESIDENT (-2)
TWS_API int tws_autotune(tws_grid* grid, int trial_steps, int* chosen);

/* Resident kernel, for small grids: the whole state (28 bytes per cell) sits
 * in the shared memory of one thread-block cluster of up to 16 SMs, and one
 * launch runs up to 4096 steps of a tws_step call, the CTAs exchanging their
 * edge rows through distributed shared memory between the phases of each
 * step.  It fits grids of up to about 8,000 cells per SM (256 x 256 fits).
 * Results are bit-identical to the tiled kernels.
 * tws_resident_fits: the cluster size (CTAs) the automatic choice gives a
 * grid of this size on the current device, or 0 if it does not fit.
 * tws_set_resident: `ctas` = TWS_RESIDENT_AUTO turns it on with the automatic
 * cluster size (one CTA for grids of at most 1024 cells, else the largest
 * power of two up to 16 that leaves every CTA a row), 1, 2, 4, 8 or 16 with
 * that many CTAs, 0 turns it off;
 * TWS_ERR_UNSUPPORTED if the grid does not fit that cluster.
 * tws_set_variant and tws_set_steps_per_launch turn it off. */
#define TWS_RESIDENT_AUTO (-1)
TWS_API int tws_resident_fits(int width, int height, int flux_storage);
TWS_API int tws_set_resident(tws_grid* grid, int ctas);

/* Advance `nsteps` steps: per step, sources, then the outflow update with
 * non-negativity scaling (flowUpdate.comp:12-63), then the depth update and
 * flow vector (flowApply.comp:13-53), fused.  Replaces the dispatch loop of
 * Terrain::PerformSimulationStep (Terrain.cpp:253-265).  Asynchronous. */
TWS_API int tws_step(tws_grid* grid, int nsteps);

/* Total water volume sum(d) * cell_area, accumulated in FP64 on the device
 * (no counterpart in the reference).  Synchronous; deterministic. */
TWS_API int tws_volume(tws_grid* grid, double* out);

/* Total water volume without allocating anything.  No counterpart in the
 * reference.
 *
 * For callers that must not allocate device memory: a renderer or game loop
 * that hands out all GPU memory from its own pools, a real-time frame path
 * that cannot afford the implicit synchronisation cudaMalloc/cudaFree may
 * cause, or code recording a CUDA graph, where allocation calls are not
 * allowed.  The caller passes the depth buffer (`pitch` floats per row, e.g.
 * from tws_get_buffers) and a device pointer `out` for the result; the call
 * only enqueues two kernels on `stream` (a cudaStream_t, NULL = legacy
 * default) and returns without waiting.  The sum is FP64, one partial per row
 * added in row order, times `cell_area`; it equals tws_volume's result to
 * within FP64 rounding (bit-identical for heights up to 1024 rows).
 *
 * Its scratch is one fixed device array of TWS_VOLUME_NOALLOC_MAX_ROWS doubles
 * (128 KB) inside libtws.so, which every GPU that loads the library holds
 * until the process exits.  Grids taller than that return
 * TWS_ERR_TOO_LARGE.  The first call on each device looks up that array's
 * device address once (cudaGetSymbolAddress) and keeps it for the life of
 * the process; make the first call before any stream capture.  A
 * cudaDeviceReset (or anything else that recreates the device's primary
 * context) after that first call is not supported: the kept address would
 * be stale.  All calls share the array and it keeps the last call's
 * partial sums (every partial is rewritten, nothing needs clearing), so two
 * calls that can run on the GPU at the same time -- on different streams,
 * or from different host threads -- race and may return wrong sums:
 * serialise them (one stream, or events).  `depth` must be 4-byte and `out`
 * 8-byte aligned (TWS_ERR_INVALID otherwise). */
#define TWS_VOLUME_NOALLOC_MAX_ROWS 16384
TWS_API int tws_volume_noalloc(const float* depth, int width, int height, int pitch,
                               double cell_area, double* out, void* stream);

/* ---- what the renderer reads ---------------------------------------------
 * The water shaders' per-texel arithmetic on the current state, written to
 * caller-owned device buffers (W x H, tightly packed; any pointer may be
 * NULL).  Replaces the reads of TerrainInfo and FlowMap in
 * waterRender.vert:21-23, waterRender.eval:32-35 and waterRender.frag:50-62,
 * 217, 240-241, 341-346 (neighbours wrap around, as the REPEAT sampler bound
 * in Terrain.cpp:313 does).  The float outputs must be 4-byte aligned
 * (TWS_ERR_INVALID otherwise); 16-byte aligned outputs and a width that is a
 * multiple of 4 take a faster path.  Asynchronous on the grid's stream. */
typedef struct tws_surface_out {
  float* height;        /* d + b                                        */
  float* render_height; /* (d + b) - 0.1, and 10 lower where d < 0.1    */
  float* normal;        /* 3 floats per cell: normalised (-dhx, 1, -dhz) */
  float* flow_speed;    /* |flow| of the RG16F flow map                 */
  float* foam;          /* saturate(|flow|^2 * 0.00004)                  */
  unsigned char* dry;   /* 1 where d < 0.1                              */
} tws_surface_out;
TWS_API int tws_surface(tws_grid* grid, const tws_surface_out* out);

/* The reference's texture layouts in caller-owned device buffers:
 * terrain_rgba = TerrainData as RGBA32F (r = terrain, g = b = 0.3, a = depth;
 * Terrain.cpp:216-220), flowmap_rg16f = FlowMap as two IEEE halves per cell
 * (flowApply.comp:7), and `mip_levels` levels of the 2x2 box-filtered mip
 * pyramid of TerrainData (Terrain.cpp:273-276), packed level after level in
 * `mips` (level l is floor(W/2^l) x floor(H/2^l) RGBA32F texels; every level
 * must be at least 1 x 1).  Any pointer may be NULL (mips need terrain_rgba).
 * terrain_rgba and mips must be 16-byte aligned and flowmap_rg16f 4-byte
 * aligned (TWS_ERR_INVALID otherwise).  The fast path (four cells per thread,
 * the first mip level written from registers) also needs flowmap_rg16f on a
 * 16-byte boundary and a width that is a multiple of 4; otherwise the call
 * runs one cell per thread, with the same results.  Asynchronous on the
 * grid's stream. */
TWS_API int tws_export_textures(tws_grid* grid, float* terrain_rgba, uint16_t* flowmap_rg16f,
                                int mip_levels, float* mips);

/* Copy state to host arrays (each may be NULL).  Flux is returned as 4 floats
 * per cell whatever the storage.  Synchronous. */
TWS_API int tws_download(tws_grid* grid, float* depth, float* flux, float* velocity);
/* Copy terrain to a host array.  Synchronous. */
TWS_API int tws_download_terrain(tws_grid* grid, float* terrain);

/* ---- asynchronous host I/O ---------------------------------------------
 * The same transfers without blocking the host, staged through device
 * buffers (52 bytes per cell, allocated on first use) and run on two copy
 * streams of the grid, so that the copies of one state overlap the steps of
 * another: upload i+1 and download i-1 run while the steps of i do.
 *
 * tws_upload_async: the state is replaced by the arrays (same arguments and
 * meaning as tws_upload) before any step queued after this call runs.
 * tws_download_async: the state as it stands after every step queued before
 * this call is copied to the arrays (same arguments as tws_download).
 * Both return at once.  The arrays must stay valid and the input arrays
 * unchanged until tws_io_wait (or tws_sync) returns, which also guarantees
 * that the output arrays hold their results.  Page-locked host arrays make
 * the copies asynchronous; with pageable ones a call may block until its
 * copy has run.  A later call of the same direction waits on the device for
 * the staging buffer of the previous one, never on the host. */
TWS_API int tws_upload_async(tws_grid* grid, const float* terrain, const float* depth,
                             const float* flux);
TWS_API int tws_download_async(tws_grid* grid, float* depth, float* flux, float* velocity);
TWS_API int tws_io_wait(tws_grid* grid);

/* Device pointers (replaces binding the textures for drawing,
 * Terrain.cpp:288, 323-330). */
TWS_API int tws_get_buffers(tws_grid* grid, tws_buffers* out);

/* ---- batches -----------------------------------------------------------
 * Many grids of different sizes advanced together: one persistent launch per
 * step covers the tiles of every member grid, and chains of 16 steps are
 * replayed from CUDA graphs.  Member grids keep their own buffers,
 * parameters and sources; while in a batch their work is ordered on the
 * batch's stream.  Grids can join and leave between calls (continuous
 * batching); each call advances every member by its own step count.  No
 * counterpart in the reference, which simulates one grid. */
typedef struct tws_batch tws_batch;

TWS_API int tws_batch_create(int flux_storage, void* stream, tws_batch** out);
TWS_API int tws_batch_destroy(tws_batch* batch); /* removes the members first */
/* The grid's queued work completes first; it must have the batch's flux storage. */
TWS_API int tws_batch_add(tws_batch* batch, tws_grid* grid);
TWS_API int tws_batch_remove(tws_batch* batch, tws_grid* grid);
TWS_API int tws_batch_size(tws_batch* batch);
/* Batched kernel variants: K steps per launch and the tile. */
TWS_API int tws_batch_variant_count(void);
TWS_API int tws_batch_variant_info(int variant, int* steps_per_launch, int* tile_x, int* tile_y);
TWS_API int tws_batch_set_variant(tws_batch* batch, int variant);
/* Times every batched variant on the members' current state (restored
 * afterwards) and keeps the fastest.  Synchronous. */
TWS_API int tws_batch_autotune(tws_batch* batch, int trial_steps, int* chosen);
/* 1 (default): replay chains from CUDA graphs; 0: launch each step directly. */
TWS_API int tws_batch_use_graphs(tws_batch* batch, int enable);
/* Every member advances `nsteps` steps.  Asynchronous. */
TWS_API int tws_batch_step(tws_batch* batch, int nsteps);
/* Member i (in the order added, removals closing the gaps) advances
 * nsteps[i] steps; n must equal tws_batch_size.  Asynchronous. */
TWS_API int tws_batch_step_each(tws_batch* batch, const int* nsteps, int n);
/* Waits for the batch and reports any member's device-side error. */
TWS_API int tws_batch_sync(tws_batch* batch);
TWS_API void* tws_batch_stream(tws_batch* batch);
TWS_API const char* tws_batch_last_error(tws_batch* batch);
/* Chains run and chains replayed from a graph so far. */
TWS_API int tws_batch_stats(tws_batch* batch, uint64_t* chains, uint64_t* graph_launches);

/* ---- serving loop ----------------------------------------------------------
 * Requests (a grid size, a synthetic scene, sources, a step count and an
 * arrival time) are admitted once their arrival time has passed and their
 * state fits the device-memory budget; admitted grids stay resident and are
 * advanced together in batch chains (continuous batching: requests join and
 * leave between chains); a finished grid reports its time to completion and
 * its FP64 water volume, and its memory is released.  No counterpart in the
 * reference (an interactive single-grid program). */
typedef struct tws_server tws_server;

typedef struct tws_server_config {
  double memory_budget_bytes; /* admission limit on resident grid state       */
  int flux_storage;           /* TWS_FLUX_* of every request                    */
  int chain_steps;            /* steps per chain; <= 0: sized per chain to about */
                              /* 1.5e9 cell-steps of work (16 to 512 steps)     */
  int batch_variant;          /* batched kernel variant; -1: autotune at start  */
  int keep_grids;             /* 1: finished grids are kept (tws_server_result  */
                              /*    returns them, the caller destroys them)     */
} tws_server_config;

typedef struct tws_request {
  uint64_t id;
  int width, height;
  uint64_t seed;       /* scene: tws_generate_scene(seed, height_scale, fill) */
  float height_scale, fill;
  tws_sim_params params;
  int nsources;
  tws_source sources[TWS_MAX_SOURCES];
  int steps;
  double arrival_s;    /* seconds after tws_server_run starts                */
} tws_request;

typedef struct tws_result {
  uint64_t id;
  int status;          /* TWS_OK, or the error that ended the request         */
  int steps;           /* steps done                                          */
  double arrival_s, admit_s, done_s; /* seconds after the run started         */
  double volume;       /* FP64 total water volume at the end                  */
  tws_grid* grid;      /* keep_grids: the finished grid, else NULL            */
} tws_result;

TWS_API int tws_server_create(const tws_server_config* config, tws_server** out);
TWS_API int tws_server_destroy(tws_server* server);
/* Thread-safe; may be called while tws_server_run is running. */
TWS_API int tws_server_submit(tws_server* server, const tws_request* request);
/* No more submissions: tws_server_run returns once everything submitted is done. */
TWS_API int tws_server_close(tws_server* server);
/* Runs the loop until the server is closed and idle (call tws_server_close
 * first, or from another thread).  serial = 1 runs the baseline instead: one
 * request at a time, in arrival order, through the single-grid path. */
TWS_API int tws_server_run(tws_server* server, int serial);
TWS_API int tws_server_result_count(tws_server* server);
TWS_API int tws_server_result(tws_server* server, int index, tws_result* out);
/* Totals of the last run: cell-steps done, wall seconds, peak resident bytes,
 * chains run. */
TWS_API int tws_server_stats(tws_server* server, double* cell_steps, double* seconds,
                             double* peak_bytes, uint64_t* chains);

/* Device bytes a grid of this size holds (tws_create's allocations). */
TWS_API double tws_grid_bytes(int width, int height, int flux_storage);

/* Block the host until the grid's queued work (asynchronous host copies
 * included) is done; reports a device-side error (TWS_ERR_TIMEOUT) raised by
 * any kernel of this grid. */
TWS_API int tws_sync(tws_grid* grid);

/* The grid's CUDA stream (cudaStream_t). */
TWS_API void* tws_stream(tws_grid* grid);

TWS_API const char* tws_error_string(int code);
TWS_API const char* tws_last_error(tws_grid* grid);

/* Number of kernels this library has launched in this process (for
 * benchmarks that report their launch count). */
TWS_API uint64_t tws_launch_count(void);

/* Library version string. */
TWS_API const char* tws_version(void);

#ifdef __cplusplus
}
#endif
#endif /* TWS_H_ */
